"""Continuum opacity with the reference's signature, on the GPU.

``build_depth_continuum`` replaces synthe_py/physics/continuum.py:73
(3-point Lagrange interpolation of log10 coefficients per continuum edge,
10**x, REAL*4 clamps) and returns (ACONT, SIGMAC) as [L, n] FP64 arrays.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from .. import _native
from ..device import DeviceAtmosphere, DeviceGrid, stream_handle


def build_depth_continuum(atmosphere, wavelength_grid, precision: str = "fp64", device="cuda"):
    if (atmosphere.continuum_wledge is None or atmosphere.continuum_abs_coeff is None
            or atmosphere.continuum_scat_coeff is None):
        raise ValueError("the atmosphere carries no continuum coefficient tables (edges, absorption, scattering)")
    lib = _native.load()
    datm = DeviceAtmosphere(atmosphere, device)
    dgrid = DeviceGrid(wavelength_grid, device=device)
    dt = torch.float64 if precision == "fp64" else torch.float32
    L = atmosphere.layers
    ca = torch.empty((L, dgrid.n), dtype=dt, device=dgrid.wavelength.device)
    cs = torch.empty((L, dgrid.n), dtype=dt, device=dgrid.wavelength.device)
    prec = _native.KS_PREC_FP64 if precision == "fp64" else _native.KS_PREC_MIXED
    _native.check(lib.ks_continuum(C.byref(datm.rec), C.byref(dgrid.rec), prec, C.c_void_p(ca.data_ptr()),
                                   C.c_void_p(cs.data_ptr()), stream_handle()))
    torch.cuda.synchronize()
    return ca.double().cpu().numpy(), cs.double().cpu().numpy()
