"""The CLI's stage files (SYNTHE_PY_STAGE_DUMPS) against the reference's own
(needs a GPU): stage 4 holds ASYNTH before the hydrogen profiles and helium
wings (engine/opacity.py:2395-2404), stage 5 the transfer's line opacity
split by FSCAT (:2416-2440, :3650-3661).  FP64 path, within 1e-11
relative of the reference's arrays (the hydrogen profile evaluates CUDA's
pow/exp/log); the .spec columns to the reference's printed precision."""

import numpy as np
import pytest

from _cases import atm_path, available_cases, case_options, gfall_path, golden, window
from kurucz_py_joss_submission_gb300 import cli

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


@pytest.mark.parametrize("name", [c for c in ("hbeta_486", "hei_447", "scat_500_501") if c in available_cases()])
def test_stage_dumps_match_reference(name, tmp_path, monkeypatch):
    g = golden(name)
    w0, w1 = window(name)
    dumps = tmp_path / "dumps"
    monkeypatch.setenv("SYNTHE_PY_STAGE_DUMPS", str(dumps))
    spec = tmp_path / "out.spec"
    opts = case_options(name)
    rc = cli.main([str(atm_path(name)), str(gfall_path(name)), "--spec", str(spec), "--wl-start", str(w0),
                   "--wl-end", str(w1), "--precision", "fp64", "--rhoxj", repr(opts["rhoxj"]),
                   "--microturb", repr(opts["microturb"])])
    assert rc == 0
    s4 = np.load(dumps / "stage_4_asynth.npz")
    s5 = np.load(dumps / "stage_5_rt.npz")
    assert rel(s4["asynth"], g["asynth"]) < 1e-11
    if "line_opacity" in g:
        assert rel(s5["line_opacity"], g["line_opacity"]) < 1e-11
    else:
        # ASYNTH (1 - FSCAT), FSCAT = exp(-RHOX / RHOXJ)
        fscat = np.exp(-np.load(atm_path(name))["depth"] / opts["rhoxj"]) if opts["rhoxj"] > 0 else 0.0
        ref = g["asynth"] * (1.0 - np.atleast_1d(fscat)[:, None])
        assert rel(s5["line_opacity"], ref) < 1e-11
    ours = np.loadtxt(spec)
    assert np.array_equal(ours[:, 0], g["spec"][:, 0])
    assert np.allclose(ours[:, 1:], g["spec"][:, 1:], rtol=1e-6, atol=0.0)
