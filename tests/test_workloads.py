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
