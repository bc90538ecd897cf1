"""The CPU oracle against the reference's own outputs (golden fixtures made
by running synthe_py itself, tests/golden/make_golden.py)."""

import numpy as np
import pytest

from _cases import available_cases, atm_path, gfall_path, golden, golden_valid, window
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
    r = oracle.synthesize(atm, cat, w0, w1, tb=tb)
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
