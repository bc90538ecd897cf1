"""The C-ABI library loads, exports every symbol of include/kurucz_gb300.h,
and its host-side functions (tables, grid, argument checks) behave.  No
compute call is made here (no GPU needed)."""

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from _cases import ROOT, available_cases, golden, window
from kurucz_py_joss_submission_gb300 import _native

HEADER = ROOT / "include" / "kurucz_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ks_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _native.load()
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_native.SIGNATURES), set(names) ^ set(_native.SIGNATURES)


def test_version():
    lib = _native.load()
    a, b = C.c_int32(), C.c_int32()
    assert lib.ks_version(C.byref(a), C.byref(b)) == 0 and a.value >= 1


def test_host_tables_match_reference(golden):
    lib = _native.load()
    ref = np.load(golden / "tables_ref.npz")
    out = [np.zeros(2001) for _ in range(3)] + [np.zeros(1001) for _ in range(2)]
    _native.check(lib.ks_get_tables(*[o.ctypes.data_as(_native.PD) for o in out]))
    for o, k in zip(out[:3], ("h0tab", "h1tab", "h2tab")):
        assert np.array_equal(o, ref[k]), k
    assert np.allclose(out[3], ref["extab"], rtol=1e-15, atol=0)
    assert np.allclose(out[4], ref["extabf"], rtol=1e-15, atol=0)


@pytest.mark.parametrize("name", available_cases())
def test_wavelength_grid_bit_exact(name):
    lib = _native.load()
    g = golden(name)
    w0, w1 = window(name)
    n = lib.ks_wavelength_grid(w0, w1, 300000.0, None, 0)
    out = np.zeros(n)
    lib.ks_wavelength_grid(w0, w1, 300000.0, out.ctypes.data_as(_native.PD), n)
    assert np.array_equal(out, g["wavelength"])


def test_full_range_grid_size():
    lib = _native.load()
    assert lib.ks_wavelength_grid(300.0, 1800.0, 300000.0, None, 0) == 537529


def test_grid_rejects_bad_resolution():
    lib = _native.load()
    assert lib.ks_wavelength_grid(500.0, 510.0, 0.0, None, 0) < 0
    assert b"positive" in lib.ks_last_error()


def test_synthesize_rejects_null_arguments():
    lib = _native.load()
    st = lib.ks_synthesize(None, None, None, None, None, 0, None, None, None, None, None)
    assert st == 1
    assert b"atmosphere" in lib.ks_last_error()


def test_workspace_size_grows_with_problem():
    lib = _native.load()
    opt = _native.KsOptions()
    a, b = C.c_size_t(), C.c_size_t()
    _native.check(lib.ks_workspace_size(1000, 72, 5941, C.byref(opt), C.byref(a)))
    _native.check(lib.ks_workspace_size(100000, 72, 5941, C.byref(opt), C.byref(b)))
    assert b.value > a.value > 0
    assert lib.ks_workspace_size(-1, 72, 10, C.byref(opt), C.byref(a)) == 1
