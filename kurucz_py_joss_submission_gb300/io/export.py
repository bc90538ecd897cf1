"""Spectrum writer (synthe_py/io/export.py:12): three columns, wavelength
(nm), F_lambda and continuum F_lambda, formatted ``%15.8f %11.6E %11.6E``."""

from __future__ import annotations

from pathlib import Path

import numpy as np


def write_spec_file(result, destination: Path) -> None:
    data = np.column_stack((result.wavelength, result.intensity, result.continuum))
    np.savetxt(destination, data, fmt="%15.8f %11.6E %11.6E")
