"""Seeded generators reproduce the line lists the golden fixtures were made from."""

import hashlib

import numpy as np
import pytest

from _cases import MG, available_cases, gfall_text, golden
from kurucz_py_joss_submission_gb300 import workloads


@pytest.mark.parametrize("name", available_cases())
def test_gfall_regenerates_bit_identically(name):
    assert hashlib.sha256(gfall_text(name).encode()).hexdigest() == str(golden(name)["gfall_sha256"])


def test_grey_atmosphere_is_hydrostatic_and_monotone():
    atm = workloads.grey_atmosphere(5800.0, 4.44)
    assert atm.rhox.size == 72
    assert np.all(np.diff(atm.rhox) > 0) and np.all(np.diff(atm.temperature) >= 0)
    # P = g * RHOX for a hydrostatic column
    assert np.allclose(atm.pressure, 10 ** 4.44 * atm.rhox, rtol=1e-12)


def test_line_draw_distributions():
    d = workloads.random_atomic_lines(50_000, 300.0, 1800.0, seed=3, log_uniform=True)
    assert np.all(np.diff(d.wavelength_nm) >= 0)
    assert d.log_gf.min() >= -8 and d.log_gf.max() <= 1
    assert abs(np.median(np.log(d.wavelength_nm)) - 0.5 * np.log(300 * 1800)) < 0.02
    assert set(np.unique(d.code)) <= set(workloads.SPECIES_CODES)


def test_band_line_draw():
    n = 120_000
    d = workloads.random_band_lines(n, 300.0, 1800.0, seed=11)
    assert d.wavelength_nm.size == n
    assert np.all(np.diff(d.wavelength_nm) >= 0)
    assert d.wavelength_nm.min() >= 300.0 and d.wavelength_nm.max() <= 1800.0
    assert np.all(d.code == workloads.BAND_CODE)
    assert d.log_gf.min() >= -8 and d.log_gf.max() <= 1
    assert abs(np.mean(d.log_gf) + 4.0) < 0.02 and abs(np.std(d.log_gf) - 1.0) < 0.02
    # E = B J (J + 1) with B in [0.3, 2] cm^-1 and J <= 150: J = 0 gives E = 0, the rest lie between
    # 2 * 0.3 and 150 * 151 * 2
    e = d.e_lower_cm
    assert e.min() >= 0.0 and e.max() <= 2.0 * 150 * 151
    assert np.all((e == 0.0) | (e >= 0.6 - 1e-12))
    # same seed, same lines
    again = workloads.random_band_lines(n, 300.0, 1800.0, seed=11)
    assert np.array_equal(again.wavelength_nm, d.wavelength_nm) and np.array_equal(again.e_lower_cm, e)


def test_band_spacing_grows_quadratically_with_j():
    """Within a band the gap between lines J and J + 1 is quadratic in J
    (third differences of the wavenumbers constant, fourth zero), as the
    dense stress case specifies -- not the linear gap of a Fortrat parabola."""
    j = np.arange(151, dtype=np.float64)
    for b in (0.3, 1.0, 2.0):
        sigma = workloads.band_wavenumbers(20000.0, b, j)
        gap = -np.diff(sigma)
        assert np.all(gap > 0) and np.all(np.diff(gap) > 0)
        assert np.allclose(np.diff(sigma, 3), -6.0 * workloads.BAND_SPACING * b, rtol=1e-6, atol=1e-9)
        # gap(J) / J^2 tends to a constant, 3 * BAND_SPACING * B (gap[149]: lines 149 -> 150)
        assert abs(gap[149] / 149.0 ** 2 / (3 * workloads.BAND_SPACING * b) - 1.0) < 0.01


def test_dense_workload_composition():
    w = workloads.WORKLOADS["dense_10m"]
    assert w["n_lines"] + w["n_band_lines"] == 10_000_000
    assert (w["teff"], w["logg"], w["wl_start"], w["wl_end"]) == (2500.0, -1.0, 300.0, 1800.0)
