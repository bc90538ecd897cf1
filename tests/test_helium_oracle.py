"""Helium lines: the oracle's restatement of the reference's helium wing pass
against the reference's He I / He II goldens, and the host rules of the C ABI
for helium lines (CPU only).

The goldens hold the reference's line opacity as the transfer sees it
(ASYNTH + AHE x STIM, engine/opacity.py:3650-3660, RHOXJ = 0); the oracle's
AHE x STIM added to the golden ASYNTH reproduces it bit for bit."""

import ctypes as C

import numpy as np
import pytest

from _cases import atm_path, available_cases, gfall_path, golden, window
from kurucz_py_joss_submission_gb300 import _native, workloads
from oracle import gfall, helium, oracle

HELIUM_CASES = [c for c in ("hei_447", "heii_468") if c in available_cases()]


def oracle_inputs(name):
    g = golden(name)
    w0, w1 = window(name)
    tb = oracle.tables()
    cat = gfall.filter_window(gfall.parse_gfall(gfall_path(name), tb["potion"]), w0, w1)
    atm = oracle.load_atmosphere(atm_path(name))
    grid = g["wavelength"]
    c = dict(wavelength=cat["wavelength"], gf=10.0 ** cat["log_gf"], elo=cat["excitation_energy"],
             gamma_rad=cat["gamma_rad"], gamma_stark=cat["gamma_stark"], gamma_vdw=cat["gamma_vdw"],
             ion_stage=cat["ion_stage"], line_type=cat["line_type"],
             center=oracle.center_indices(grid, cat["wavelength"]))
    return g, c, atm, grid


@pytest.mark.parametrize("name,ltype,ion", [("hei_447", -3, 1), ("heii_468", -6, 2)])
def test_oracle_line_opacity_bit_exact(name, ltype, ion):
    if name not in HELIUM_CASES:
        pytest.skip("golden missing")
    g, c, atm, grid = oracle_inputs(name)
    rows = helium.helium_rows(c)
    assert rows.size == 1 and c["line_type"][rows[0]] == ltype and c["ion_stage"][rows[0]] == ion
    he = helium.line_opacity(c, atm, grid, g["cont_abs"] + g["cont_scat"])
    assert np.count_nonzero(he) > 1000
    assert np.array_equal(g["asynth"] + he, g["line_opacity"])


def test_oracle_detects_planted_error():
    g, c, atm, grid = oracle_inputs(HELIUM_CASES[0])
    bad = dict(c, gamma_stark=c["gamma_stark"].copy())
    bad["gamma_stark"][helium.helium_rows(c)[0]] *= 1.01   # 1 % on the He line's Stark width
    he = helium.line_opacity(bad, atm, grid, g["cont_abs"] + g["cont_scat"])
    assert not np.array_equal(g["asynth"] + he, g["line_opacity"])


def test_helium_lines_table():
    d = workloads.helium_lines(400.0, 510.0)
    assert len(d) == 6 and set(d.code) == {2.00, 2.01}
    assert d.n_lower is None and d.n_upper is None   # no NBLO/NBUP: no fort.19 route


def _lines_record(n_lines, n_helium):
    dummy = C.c_void_p(16)   # never dereferenced: the checks read the record only
    rec = _native.KsLines()
    rec.n_lines = n_lines
    for name, typ in _native.KsLines._fields_:
        if typ is _native.P:
            setattr(rec, name, dummy.value)
    rec.sorted_by_wavelength = 1
    rec.n_helium = n_helium
    return rec


def test_batch_takes_helium_lines():
    # the lines pass the batch's checks (the call fails on the missing jobs)
    L = _native.load(build_if_missing=False)
    size = C.c_size_t(0)
    rec = _lines_record(10, 1)
    assert L.ks_batch_workspace_size(C.byref(rec), None, 0, None, C.byref(size)) == _native.KS_ERR_INVALID
    assert b"no jobs" in L.ks_last_error()
    rec = _lines_record(10, 11)
    assert L.ks_batch_workspace_size(C.byref(rec), None, 0, None, C.byref(size)) == _native.KS_ERR_INVALID
    assert b"n_helium" in L.ks_last_error()
