"""Per-wavelength LTE transfer with the reference's signature, on the GPU.

``solve_lte_spectrum`` replaces synthe_py/engine/radiative.py:282: one JOSH
solve for the continuum and one for continuum + lines per wavelength
(physics/josh_solver.py:367), F_nu at the surface.  One GPU thread handles
one wavelength's depth column; ``n_workers`` is accepted for signature
compatibility and ignored.
"""

from __future__ import annotations

import ctypes as C
from typing import Optional, Tuple

import numpy as np
import torch

from .. import _native
from ..device import DeviceAtmosphere, DeviceGrid, stream_handle
from ..io.atmosphere import AtmosphereModel


def solve_lte_spectrum(
    wavelength_nm: np.ndarray,
    temperature: np.ndarray,
    column_mass: np.ndarray,
    cont_abs: np.ndarray,
    cont_scat: np.ndarray,
    line_opacity: np.ndarray,
    line_scattering: np.ndarray,
    line_source: Optional[np.ndarray] = None,
    n_workers: Optional[int] = None,
    precision: str = "fp64",
    device="cuda",
    stats: Optional[dict] = None,
) -> Tuple[np.ndarray, np.ndarray]:
    lib = _native.load()
    L = int(np.asarray(temperature).size)
    T = np.asarray(temperature, np.float64)
    atm = AtmosphereModel(
        depth=np.asarray(column_mass, np.float64), temperature=T,
        gas_pressure=np.zeros(L), electron_density=np.zeros(L), mass_density=np.ones(L),
        turbulent_velocity=np.zeros(L), hckt=1.4388 / np.maximum(T, 1.0),
        population_per_ion=np.zeros((L, 1, 1)), doppler_per_ion=np.zeros((L, 1, 1)),
    )
    datm = DeviceAtmosphere(atm, device)
    dgrid = DeviceGrid(wavelength_nm, device=device)
    dev = dgrid.wavelength.device
    dt = torch.float64 if precision == "fp64" else torch.float32
    npdt = np.float64 if precision == "fp64" else np.float32

    def up(a):
        return torch.from_numpy(np.ascontiguousarray(a, npdt)).to(dev) if a is not None else None

    ca, cs, lo, ls, src = up(cont_abs), up(cont_scat), up(line_opacity), up(line_scattering), up(line_source)
    ft = torch.empty(dgrid.n, dtype=torch.float64, device=dev)
    fc = torch.empty(dgrid.n, dtype=torch.float64, device=dev)
    prec = _native.KS_PREC_FP64 if precision == "fp64" else _native.KS_PREC_MIXED
    st = _native.KsStats()

    def p(t):
        return C.c_void_p(t.data_ptr()) if t is not None else None

    _native.check(lib.ks_formal_solution(C.byref(datm.rec), C.byref(dgrid.rec), prec, p(ca), p(cs), p(lo),
                                         p(ls), p(src), p(ft), p(fc), C.byref(st), stream_handle()))
    torch.cuda.synchronize()
    if stats is not None:
        stats.update(st.as_dict())
    return ft.cpu().numpy(), fc.cpu().numpy()
