"""fort.19 NORMAL lines (metal lines with NBLO/NBUP set): the oracle's
restatement of _add_fort19_asynth (engine/opacity.py:1335-1488) against the
reference's golden, and the host rules of the C ABI for these lines (CPU
only).  The golden's ASYNTH holds the reference's fort.19 profiles; the
oracle's own ASYNTH (without those lines, which leave TRANSP) plus its
fort.19 term reproduces it to the rounding of the ASYNTH sums."""

import ctypes as C

import numpy as np
import pytest

from _cases import atm_path, available_cases, gfall_path, golden, window
from kurucz_py_joss_submission_gb300 import _native
from kurucz_py_joss_submission_gb300.io.lines import atomic
from oracle import fort19, gfall, oracle

CASE = "fort19_500_501"
pytestmark = pytest.mark.skipif(CASE not in available_cases(), reason="golden missing")


def test_oracle_asynth_with_fort19_lines():
    g = golden(CASE)
    w0, w1 = window(CASE)
    tb = oracle.tables()
    cat = gfall.filter_window(gfall.parse_gfall(gfall_path(CASE), tb["potion"]), w0, w1)
    rows = fort19.normal_rows(cat)
    assert rows.size >= 30
    r = oracle.synthesize(oracle.load_atmosphere(atm_path(CASE)), cat, w0, w1, tb=tb)
    rel = np.abs(r["asynth"] - g["asynth"]) / np.maximum(np.abs(g["asynth"]), 1e-300)
    assert float(rel.max()) < 1e-13
    # the fort.19 lines carry a visible part of it
    term = fort19.asynth_term(dict(cat, center=oracle.center_indices(g["wavelength"], cat["wavelength"])),
                              oracle.load_atmosphere(atm_path(CASE)), g["wavelength"],
                              g["cont_abs"] + g["cont_scat"])
    assert np.count_nonzero(term) > 10000


@pytest.mark.skipif("aut_500_501" not in available_cases(), reason="golden missing")
def test_oracle_asynth_with_autoionizing_lines():
    name = "aut_500_501"
    g = golden(name)
    w0, w1 = window(name)
    tb = oracle.tables()
    cat = gfall.filter_window(gfall.parse_gfall(gfall_path(name), tb["potion"]), w0, w1)
    assert fort19.aut_rows(cat).size >= 20
    gs = cat["gamma_stark_log"][fort19.aut_rows(cat)]
    assert np.any(gs > 0) and np.any(gs < 0)   # ASHORE of both signs
    r = oracle.synthesize(oracle.load_atmosphere(atm_path(name)), cat, w0, w1, tb=tb)
    rel = np.abs(r["asynth"] - g["asynth"]) / np.maximum(np.abs(g["asynth"]), 1e-300)
    assert float(rel.max()) < 1e-13


@pytest.mark.skipif("cont_505_507" not in available_cases(), reason="golden missing")
def test_oracle_asynth_with_merged_continuum_records():
    name = "cont_505_507"
    g = golden(name)
    w0, w1 = window(name)
    tb = oracle.tables()
    cat = gfall.filter_window(gfall.parse_gfall(gfall_path(name), tb["potion"]), w0, w1)
    rows = fort19.cont_rows(cat)
    assert rows.size == 3 and np.all(cat["xjp"][rows] > 3)
    r = oracle.synthesize(oracle.load_atmosphere(atm_path(name)), cat, w0, w1, tb=tb)
    rel = np.abs(r["asynth"] - g["asynth"]) / np.maximum(np.abs(g["asynth"]), 1e-300)
    assert float(rel.max()) < 1e-13


@pytest.mark.parametrize("name,key", [("ncon_252", "asynth"), ("heii_595", "line_opacity")])
def test_oracle_continuum_merge_limits(name, key):
    """fort.19 records with NCON set: the WCON cut and the WTAIL taper of a
    NORMAL line's wings (Mg I, NCON 2) and of a helium line's (He II, NCON 5)."""
    if name not in available_cases():
        pytest.skip("golden missing")
    g = golden(name)
    w0, w1 = window(name)
    tb = oracle.tables()
    cat = gfall.filter_window(gfall.parse_gfall(gfall_path(name), tb["potion"]), w0, w1)
    assert np.any(cat["iso2"] > 0)
    r = oracle.synthesize(oracle.load_atmosphere(atm_path(name)), cat, w0, w1, tb=tb)
    mine = r["line_opacity"] if key == "line_opacity" else r["asynth"]
    rel = np.abs(mine - g[key]) / np.maximum(np.abs(g[key]), 1e-300)
    assert float(rel.max()) < 1e-13


def test_oracle_detects_planted_error():
    g = golden(CASE)
    w0, w1 = window(CASE)
    tb = oracle.tables()
    cat = gfall.filter_window(gfall.parse_gfall(gfall_path(CASE), tb["potion"]), w0, w1)
    cat = dict(cat, center=oracle.center_indices(g["wavelength"], cat["wavelength"]))
    atm = oracle.load_atmosphere(atm_path(CASE))
    good = fort19.asynth_term(cat, atm, g["wavelength"], g["cont_abs"] + g["cont_scat"])
    bad_cat = dict(cat, gamma_vdw=cat["gamma_vdw"] * 1.5)   # damping constants off by 50 %
    bad = fort19.asynth_term(bad_cat, atm, g["wavelength"], g["cont_abs"] + g["cont_scat"])
    assert not np.array_equal(good, bad)


def test_reader_fields_and_routing():
    w0, w1 = window(CASE)
    cat = atomic.load_catalog_window(gfall_path(CASE), w0, w1)
    nb = (cat.n_lower != 0) | (cat.n_upper != 0)
    assert nb.sum() >= 30 and np.all(cat.process_mask[nb] == 0)   # they leave TRANSP
    assert np.all(cat.iso1 == 0) and np.all(cat.iso2 == 0)
    assert np.all(cat.gamma_rad_log[nb] != 0.0)   # the logs as read


def test_batch_takes_fort19_lines():
    L = _native.load(build_if_missing=False)
    dummy = C.c_void_p(16)
    rec = _native.KsLines()
    rec.n_lines = 10
    for name, typ in _native.KsLines._fields_:
        if typ is _native.P:
            setattr(rec, name, dummy.value)
    rec.sorted_by_wavelength = 1
    rec.n_f19 = 1
    size = C.c_size_t(0)
    # the lines pass the batch's checks (the call fails on the missing jobs)
    assert L.ks_batch_workspace_size(C.byref(rec), None, 0, None, C.byref(size)) == _native.KS_ERR_INVALID
    assert b"no jobs" in L.ks_last_error()
