"""The native gfall reader against the oracle's restatement of
synthe_py/io/lines/atomic.py:299 (window, routing, defaults)."""

import numpy as np
import pytest

from _cases import SMALL_CASES, gfall_path, window
from kurucz_py_joss_submission_gb300.io.lines import atomic
from oracle import gfall, oracle


@pytest.fixture(scope="module")
def potion():
    return oracle.tables()["potion"]


@pytest.mark.parametrize("name", SMALL_CASES)
def test_reader_matches_oracle(name, potion):
    w0, w1 = window(name)
    a = atomic.load_catalog_window(gfall_path(name), w0, w1)
    o = gfall.filter_window(gfall.parse_gfall(gfall_path(name), potion), w0, w1)
    r = gfall.routing(o)
    assert len(a) == o["wavelength"].size
    for k, v in [("wavelength", o["wavelength"]), ("gamma_rad", o["gamma_rad"]),
                 ("gamma_stark", o["gamma_stark"]), ("gamma_vdw", o["gamma_vdw"]),
                 ("excitation_energy", o["excitation_energy"])]:
        assert np.array_equal(getattr(a, k), v), k
    # 10**log_gf: NumPy's vectorised pow and libm's may differ in the last bit
    assert np.allclose(a.gf, r["gf"], rtol=1e-15, atol=0)
    assert np.allclose(a.cgf, r["cgf"], rtol=1e-15, atol=0)
    for k, v in [("element_idx", r["element_idx"]), ("ion_stages", o["ion_stage"]),
                 ("process_mask", r["process_mask"]), ("asynth_mask", r["asynth_mask"])]:
        assert np.array_equal(getattr(a, k), v), k


def test_damping_defaults(tmp_path, potion):
    line = ("   500.0058 -2.338 26.01   31700.754  1.0 SYNTH        51700.521  2.0 SYNTH "
            "      0.00  0.00  0.00" + " " * 62)
    p = tmp_path / "d.gf"
    p.write_text(line + "\n")
    a = atomic.load_catalog(p)
    o = gfall.parse_gfall(p, potion)
    for k in ("gamma_rad", "gamma_stark", "gamma_vdw"):
        assert np.allclose(getattr(a, k), o[k], rtol=1e-15), k
    assert a.gamma_rad[0] > 0 and a.gamma_stark[0] > 0 and a.gamma_vdw[0] > 0


def test_special_classes_and_window(tmp_path, potion):
    base = "   500.0058 -2.338 {code}   31700.754  1.0 SYNTH        51700.521  2.0 SYNTH       8.00 -5.50 -7.50"
    rows = [base.format(code=c) + " " * 62 for c in ("26.00", " 1.00", " 2.00", " 2.01", "93.00")]
    p = tmp_path / "s.gf"
    p.write_text("\n".join(rows) + "\n# comment\n\n")
    a = atomic.load_catalog(p)
    assert list(a.line_types) == [0, -1, -3, -6, 0]
    assert list(a.process_mask) == [1, 0, 1, 1, 0]      # H skipped, Z>92 unknown
    assert list(a.asynth_mask) == [1, 0, 1, 1, 1]
    assert list(a.element_idx) == [25, 0, 1, 1, -1]
    # window: the line sits at 1e7/(51700.521-31700.754) = 500.0058 nm
    assert len(atomic.load_catalog_window(p, 600.0, 601.0)) == 1   # only H (100 nm margin)
    assert len(atomic.load_catalog_window(p, 500.1, 501.0)) == 5   # within 0.1 nm margin


def test_missing_file_raises(tmp_path):
    with pytest.raises(FileNotFoundError):
        atomic.load_catalog(tmp_path / "nope.gf")


def test_whitespace_records(tmp_path):
    p = tmp_path / "w.gf"
    p.write_text("500.1 Fe 1 -1.5 20000.0 1e-8 1e-22 1e-24\n500.2 He 1 -1.0 0.0 1e-8 1e-22\n")
    a = atomic.load_catalog(p)
    assert len(a) == 2
    assert list(a.element_idx) == [25, 1] and list(a.line_types) == [0, -3]
