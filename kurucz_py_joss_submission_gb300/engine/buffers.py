"""Result record of a synthesis (synthe_py/engine/buffers.py:37 SynthResult)."""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict

import numpy as np


@dataclass
class SynthResult:
    wavelength: np.ndarray
    intensity: np.ndarray      # F_lambda (erg s^-1 cm^-2 nm^-1 per the reference's units)
    continuum: np.ndarray      # continuum F_lambda
    timings: Dict[str, float] = field(default_factory=dict)
    stats: Dict[str, int] = field(default_factory=dict)
