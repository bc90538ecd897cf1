"""Hydrogen line opacity: the oracle's HPROF4 restatement against the
reference's Balmer-line goldens, and the host-side rules of the C ABI for
hydrogen lines (CPU only).

The goldens hold the reference's line opacity as the transfer sees it
(ASYNTH + AHLINE, engine/opacity.py:2465-2503, RHOXJ = 0); the oracle's
AHLINE added to the golden ASYNTH reproduces it bit for bit."""

import ctypes as C

import numpy as np
import pytest

from _cases import atm_path, available_cases, gfall_path, golden, window
from kurucz_py_joss_submission_gb300 import _native, workloads
from oracle import gfall, hydrogen, oracle

HYDROGEN_CASES = [c for c in ("hbeta_486", "hgamma_434") if c in available_cases()]


def oracle_inputs(name):
    g = golden(name)
    w0, w1 = window(name)
    tb = oracle.tables()
    cat = gfall.filter_window(gfall.parse_gfall(gfall_path(name), tb["potion"]), w0, w1)
    atm = oracle.load_atmosphere(atm_path(name))
    grid = g["wavelength"]
    c = dict(wavelength=cat["wavelength"], gf=10.0 ** cat["log_gf"], elo=cat["excitation_energy"],
             n_lower=cat["n_lower"], n_upper=cat["n_upper"], line_type=cat["line_type"],
             ion_stage=cat["ion_stage"], center=oracle.center_indices(grid, cat["wavelength"]))
    return g, c, atm, grid


@pytest.mark.parametrize("name", HYDROGEN_CASES)
def test_oracle_line_opacity_bit_exact(name):
    g, c, atm, grid = oracle_inputs(name)
    hyd = (np.isin(c["line_type"], (-1, -2))) & (c["ion_stage"] == 1)
    assert hyd.sum() == 3 and set(c["n_upper"][hyd]) == {4, 5, 6} and set(c["n_lower"][hyd]) == {2}
    ah = hydrogen.line_opacity(c, atm, grid, g["cont_abs"] + g["cont_scat"])
    assert np.count_nonzero(ah) > 1000
    assert np.array_equal(g["asynth"] + ah, g["line_opacity"])


def test_oracle_detects_planted_error():
    g, c, atm, grid = oracle_inputs(HYDROGEN_CASES[0])
    hyd = np.flatnonzero(np.isin(c["line_type"], (-1, -2)) & (c["ion_stage"] == 1))
    inside = hyd[(c["wavelength"][hyd] > grid[0]) & (c["wavelength"][hyd] < grid[-1])]
    assert inside.size == 1   # H beta; the other two lie far outside the window
    bad = dict(c, n_upper=c["n_upper"].copy())
    bad["n_upper"][inside[0]] += 1   # a wrong upper level on the window's Balmer line
    ah = hydrogen.line_opacity(bad, atm, grid, g["cont_abs"] + g["cont_scat"])
    assert not np.array_equal(g["asynth"] + ah, g["line_opacity"])


def test_balmer_lines_carry_levels():
    d = workloads.balmer_lines([3, 4, 5])
    lo, up = d.levels()
    assert list(lo) == [2, 2, 2] and list(up) == [3, 4, 5]
    assert np.all(np.diff(np.sort(d.wavelength_nm)) > 0)


def _lines_record(n_lines, n_hydrogen):
    dummy = C.c_void_p(16)   # never dereferenced: the checks read the record only
    rec = _native.KsLines()
    rec.n_lines = n_lines
    for name, typ in _native.KsLines._fields_:
        if typ is _native.P:
            setattr(rec, name, dummy.value)
    rec.sorted_by_wavelength = 1
    rec.n_hydrogen = n_hydrogen
    return rec


def test_batch_takes_hydrogen_lines():
    # the lines pass the batch's checks (the call fails on the missing jobs);
    # each job's hydrogen lines are found when the plan is made
    L = _native.load(build_if_missing=False)
    rec = _lines_record(10, 1)
    size = C.c_size_t(0)
    st = L.ks_batch_workspace_size(C.byref(rec), None, 0, None, C.byref(size))
    assert st == _native.KS_ERR_INVALID
    assert b"no jobs" in L.ks_last_error()
    rec = _lines_record(10, 11)   # more hydrogen lines than lines
    assert L.ks_batch_workspace_size(C.byref(rec), None, 0, None, C.byref(size)) == _native.KS_ERR_INVALID


def test_hydrogen_tables_validated():
    L = _native.load(build_if_missing=False)
    t = _native.KsHydrogenTables()
    assert L.ks_init_hydrogen_tables(C.byref(t)) == _native.KS_ERR_INVALID
    _native._init_hydrogen_tables(L)   # the package's tables are accepted
