"""Synthesis driver (synthe_py.engine re-exports run_synthesis)."""

from .opacity import run_synthesis  # noqa: F401
