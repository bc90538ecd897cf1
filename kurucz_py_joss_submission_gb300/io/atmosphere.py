"""Converted-atmosphere (.npz) reader, the fields the synthesis path uses.

Mirrors synthe_py/io/atmosphere.py:17 (AtmosphereModel) and :82
(load_cached): the same key names and fallbacks (depth|rhox|qrhox, ...).
"""

from __future__ import annotations

from dataclasses import dataclass, field
from pathlib import Path
from typing import Dict, Optional

import numpy as np


@dataclass
class AtmosphereModel:
    depth: np.ndarray
    temperature: np.ndarray
    gas_pressure: np.ndarray
    electron_density: np.ndarray
    mass_density: np.ndarray
    turbulent_velocity: np.ndarray
    metadata: Dict[str, object] = field(default_factory=dict)
    hckt: Optional[np.ndarray] = None
    xnf_h: Optional[np.ndarray] = None
    xnf_he1: Optional[np.ndarray] = None
    xnf_h2: Optional[np.ndarray] = None
    population_per_ion: Optional[np.ndarray] = None
    doppler_per_ion: Optional[np.ndarray] = None
    continuum_wledge: Optional[np.ndarray] = None
    continuum_half_edge: Optional[np.ndarray] = None
    continuum_delta_edge: Optional[np.ndarray] = None
    continuum_abs_coeff: Optional[np.ndarray] = None
    continuum_scat_coeff: Optional[np.ndarray] = None
    continuum_coeff_log10: bool = False

    @property
    def layers(self) -> int:
        return int(self.temperature.size)


def _pick(data, *names, required=True):
    for n in names:
        if n in data:
            return np.asarray(data[n])
    if required:
        raise KeyError(f"Required atmosphere field missing: {' / '.join(names)}")
    return None


def load_cached(path: Path) -> AtmosphereModel:
    """Load a converted atmosphere (.npz written by convert_atm_to_npz)."""
    with np.load(path, allow_pickle=False) as d:
        temperature = np.asarray(_pick(d, "temperature", "qt"), dtype=np.float64)
        hckt = d["hckt"] if "hckt" in d else (d["qhckt"] if "qhckt" in d else None)
        if hckt is None:
            # populations.py:166-170 fallback: hc/k = 1.4388 cm K
            hckt = 1.4388 / np.maximum(temperature, 1.0)
        xnf_he1 = d["xnf_he1"] if "xnf_he1" in d else None
        if xnf_he1 is None and "qxnf_he" in d:
            he = np.asarray(d["qxnf_he"])
            xnf_he1 = he[:, 0] if he.ndim == 2 else None
        atm = AtmosphereModel(
            depth=np.asarray(_pick(d, "depth", "rhox", "qrhox"), dtype=np.float64),
            temperature=temperature,
            gas_pressure=np.asarray(_pick(d, "gas_pressure", "qp"), dtype=np.float64),
            electron_density=np.asarray(_pick(d, "electron_density", "qxne"), dtype=np.float64),
            mass_density=np.asarray(_pick(d, "mass_density", "qrho"), dtype=np.float64),
            turbulent_velocity=np.asarray(_pick(d, "turbulent_velocity", "qvturb"), dtype=np.float64),
            hckt=np.asarray(hckt, dtype=np.float64),
            xnf_h=np.asarray(_pick(d, "xnf_h", "qxnf_h", required=False), dtype=np.float64)
            if ("xnf_h" in d or "qxnf_h" in d) else None,
            xnf_he1=np.asarray(xnf_he1, dtype=np.float64) if xnf_he1 is not None else None,
            xnf_h2=np.asarray(_pick(d, "xnf_h2", "qxnf_h2", required=False), dtype=np.float64)
            if ("xnf_h2" in d or "qxnf_h2" in d) else None,
            population_per_ion=np.asarray(d["population_per_ion"], dtype=np.float64)
            if "population_per_ion" in d else None,
            doppler_per_ion=np.asarray(d["doppler_per_ion"], dtype=np.float64)
            if "doppler_per_ion" in d else None,
            continuum_wledge=np.asarray(d["wledge"], dtype=np.float64) if "wledge" in d else None,
            continuum_half_edge=np.asarray(d["half_edge"], dtype=np.float64) if "half_edge" in d else None,
            continuum_delta_edge=np.asarray(d["delta_edge"], dtype=np.float64) if "delta_edge" in d else None,
            continuum_abs_coeff=np.asarray(d["cont_abs_coeff"], dtype=np.float64) if "cont_abs_coeff" in d else None,
            continuum_scat_coeff=np.asarray(d["cont_scat_coeff"], dtype=np.float64) if "cont_scat_coeff" in d else None,
            continuum_coeff_log10=bool(d["cont_coeff_log10"]) if "cont_coeff_log10" in d else False,
        )
        for k in ("teff", "glog"):
            if k in d:
                atm.metadata[k] = float(np.asarray(d[k]).item())
    return atm
