"""Helpers shared by the tests: golden cases, catalogs and oracle runs."""

from __future__ import annotations

import functools
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(GOLDEN))

import make_golden as MG  # noqa: E402  (case table; never runs the reference here)

from kurucz_py_joss_submission_gb300 import workloads  # noqa: E402

SMALL_CASES = ["tiny_500_501", "uv_300_302", "strong_600_601"]


def available_cases():
    return [c for c in MG.CASES if (GOLDEN / f"case_{c}.npz").exists()]


@functools.lru_cache(maxsize=None)
def gfall_path(name: str) -> Path:
    case = MG.CASES[name]
    p = Path("/tmp") / f"kgb300_case_{name}.gf"
    text = workloads.format_gfall(MG.case_lines(case))
    p.write_text(text)
    return p


def gfall_text(name: str) -> str:
    return workloads.format_gfall(MG.case_lines(MG.CASES[name]))


def golden(name: str):
    return np.load(GOLDEN / f"case_{name}.npz")


def golden_valid(g) -> np.ndarray:
    shape = tuple(g["valid_shape"])
    return np.unpackbits(g["valid_mask"])[: int(np.prod(shape))].reshape(shape).astype(bool)


def atm_path(name: str) -> Path:
    return GOLDEN / f"atm_{MG.CASES[name]['atm']}.npz"


def window(name: str):
    c = MG.CASES[name]
    return c["wl_start"], c["wl_end"]


def case_options(name: str) -> dict:
    """Synthesis options of a case besides the window: line scattering scale
    (``--rhoxj``) and microturbulence (``--microturb``, km/s)."""
    c = MG.CASES[name]
    return {"rhoxj": float(c.get("rhoxj", 0.0)), "microturb": float(c.get("microturb", 0.0))}


def device_options(name: str) -> dict:
    """The same options as ``make_options`` keywords."""
    o = case_options(name)
    return {"rhoxj": o["rhoxj"], "microturb_kms": o["microturb"]}
