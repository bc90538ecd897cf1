"""The CPU oracle against the reference's own outputs (golden fixtures made
by running synthe_py itself, tests/golden/make_golden.py)."""

import numpy as np
import pytest

from _cases import available_cases, atm_path, case_options, gfall_path, golden, golden_valid, window
from oracle import gfall, oracle


@pytest.fixture(scope="module")
def tb():
    return oracle.tables()


def rel(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def test_tables_match_reference(tb, golden):
    ref = np.load(golden / "tables_ref.npz")
    for k in ("h0tab", "h1tab", "h2tab"):
        assert np.array_equal(tb[k], ref[k]), k
    assert np.allclose(tb["extab"], ref["extab"], rtol=1e-15, atol=0)
    assert np.allclose(tb["extabf"], ref["extabf"], rtol=1e-15, atol=0)


@pytest.mark.parametrize("name", available_cases())
def test_oracle_against_reference(name, tb):
    g = golden(name)
    w0, w1 = window(name)
    cat = gfall.filter_window(gfall.parse_gfall(gfall_path(name), tb["potion"]), w0, w1)
    atm = oracle.load_atmosphere(atm_path(name))
    r = oracle.synthesize(atm, cat, w0, w1, tb=tb, **case_options(name))
    # bins and gates are exact
    assert np.array_equal(r["wavelength"], g["wavelength"])
    assert np.array_equal(r["center_indices"], g["line_indices"])
    assert np.array_equal(r["valid_mask"], golden_valid(g))
    if "transp" in g:
        assert rel(r["transp"], g["transp"]) < 1e-13
        assert rel(r["asynth"], g["asynth"]) < 1e-13
        assert rel(r["cont_abs"], g["cont_abs"]) < 1e-13
        assert rel(r["cont_scat"], g["cont_scat"]) < 1e-13
    else:
        pairs = g["transp_pairs"]
        assert rel(r["transp"][pairs[:, 0], pairs[:, 1]], g["transp_values"]) < 1e-13
        rows = g["asynth_rows"]
        assert rel(r["asynth"][rows], g["asynth"]) < 1e-12
        assert rel(r["cont_abs"][rows], g["cont_abs_rows"]) < 1e-13
    if "line_opacity" in g:
        # hydrogen lines: ASYNTH + AHLINE (bit for bit on the golden ASYNTH
        # and continuum, test_hydrogen_oracle.py; here on the oracle's own)
        assert rel(r["line_opacity"], g["line_opacity"]) < 1e-12
    assert rel(r["flux_total_hz"], g["flux_total_hz"]) < 1e-12
    assert rel(r["flux_cont_hz"], g["flux_cont_hz"]) < 1e-12


def test_strong_case_reaches_maxj_path(tb):
    name = "strong_600_601"
    w0, w1 = window(name)
    cat = gfall.filter_window(gfall.parse_gfall(gfall_path(name), tb["potion"]), w0, w1)
    r = oracle.synthesize(oracle.load_atmosphere(atm_path(name)), cat, w0, w1, tb=tb)
    assert (r["iterations"][:, 1] < 0).sum() > 10


def test_oracle_detects_planted_error(tb):
    """A mistake planted in the oracle's inputs must show up against the golden."""
    name = "tiny_500_501"
    g = golden(name)
    w0, w1 = window(name)
    cat = gfall.filter_window(gfall.parse_gfall(gfall_path(name), tb["potion"]), w0, w1)
    cat["log_gf"] = cat["log_gf"] + 0.01  # every line 2.3% stronger
    r = oracle.synthesize(oracle.load_atmosphere(atm_path(name)), cat, w0, w1, tb=tb)
    assert rel(r["asynth"], g["asynth"]) > 1e-6


def test_tabi_case_hits_rounding_ties(tb):
    """The tabi_500_501 fixture exercises the reference's incremental TABI
    (line_opacity.py:540-548) where it matters: near-wing offsets inside the
    evaluated wing of valid Fe/Ti pairs at which int(0.5 + n*TABSTEP) and the
    incremental sum's integer part differ.  (np.cumsum adds sequentially, as
    the reference's loop does.)"""
    name = "tabi_500_501"
    g = golden(name)
    w0, w1 = window(name)
    cat = gfall.filter_window(gfall.parse_gfall(gfall_path(name), tb["potion"]), w0, w1)
    atm = oracle.load_atmosphere(atm_path(name))
    r = oracle.synthesize(atm, cat, w0, w1, tb=tb)
    grid = g["wavelength"]
    resolu = 1.0 / (grid[1] / grid[0] - 1.0)
    valid = golden_valid(g)
    ties = 0
    for li in np.nonzero(np.isin(cat["nelem"], [22, 26]) & (cat["line_type"] == 0))[0]:
        lw = cat["wavelength"][li]
        for d in np.nonzero(valid[li])[0]:
            dop = atm["doppler_per_ion"][d, cat["ion_stage"][li] - 1, cat["nelem"][li] - 1]
            dopple = (dop * lw) / lw
            dvoigt = 1.0 / (dopple * resolu)
            ts = 200.0 * dvoigt
            n = min(int(10.0 * dopple * resolu), int(r["reach"][li, d]), int(10.0 / dvoigt))
            if n < 1:
                continue
            k = np.arange(1, n + 1, dtype=np.float64)
            inc = np.cumsum(np.concatenate([[0.5], np.full(n, ts)]))[1:]
            ties += int(np.sum(inc.astype(np.int64) != (0.5 + k * ts).astype(np.int64)))
    assert ties > 0
