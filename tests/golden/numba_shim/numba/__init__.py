"""Identity stand-in for ``numba`` so the pure-Python reference runs without it.

Test infrastructure only: ``make_golden.py`` puts this directory first on
``PYTHONPATH`` when it runs the reference pipeline to produce golden fixtures.
``jit``/``njit`` return the function unchanged and ``prange`` is ``range``, so
the reference executes its kernels as plain Python with NumPy semantics.
"""

from __future__ import annotations


def _identity_decorator(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def wrap(fn):
        return fn

    return wrap


jit = _identity_decorator
njit = _identity_decorator
vectorize = _identity_decorator
guvectorize = _identity_decorator
prange = range


def get_num_threads() -> int:
    return 1


def set_num_threads(n: int) -> None:  # noqa: ARG001
    return None


class _Types:
    def __getattr__(self, name):
        return object


types = _Types()
config = _Types()
