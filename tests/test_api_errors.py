"""Error behaviour of the Python mirror of the reference API: the same
exception types as synthe_py for the same bad inputs
(physics/line_opacity.py:685, engine/opacity.py:531,
physics/continuum.py:292), raised before any device work (CPU only)."""

from dataclasses import replace
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest

from kurucz_py_joss_submission_gb300.engine import continuum
from kurucz_py_joss_submission_gb300.engine.opacity import _build_wavelength_grid
from kurucz_py_joss_submission_gb300.io import atmosphere as atm_io
from kurucz_py_joss_submission_gb300.physics.line_opacity import compute_transp

ATM = Path(__file__).parent / "golden" / "atm_t5800g444.npz"


def test_compute_transp_needs_continuum_and_grid():
    atm = atm_io.load_cached(ATM)
    grid = np.linspace(500.0, 501.0, 11)
    with pytest.raises(ValueError):
        compute_transp(None, None, atm, 1e-3, None, grid)
    with pytest.raises(ValueError):
        compute_transp(None, None, atm, 1e-3, np.ones((atm.layers, 11)), None)


@pytest.mark.parametrize("resolution", [0.0, -300000.0])
def test_grid_needs_positive_resolution(resolution):
    cfg = SimpleNamespace(wavelength_grid=SimpleNamespace(start=500.0, end=510.0, resolution=resolution))
    with pytest.raises(ValueError):
        _build_wavelength_grid(cfg)


def test_continuum_needs_coefficient_tables():
    atm = replace(atm_io.load_cached(ATM), continuum_abs_coeff=None)
    with pytest.raises(ValueError):
        continuum.build_depth_continuum(atm, np.linspace(500.0, 501.0, 11))
