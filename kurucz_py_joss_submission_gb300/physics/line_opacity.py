"""TRANSP and ASYNTH with the reference's signatures, computed on the GPU.

``compute_transp`` replaces synthe_py/physics/line_opacity.py:620 and
``compute_asynth_from_transp`` replaces :946.  Both take host arrays, run the
FP64 kernels through the C ABI and return host arrays in catalog order, so
code written against the reference's seams runs unchanged.  The fused fast
path is ``device.Synthesizer``.
"""

from __future__ import annotations

import ctypes as C
from typing import Optional, Tuple

import numpy as np
import torch

from .. import _native
from ..device import DeviceAtmosphere, DeviceCatalog, DeviceGrid, make_options, stream_handle
from ..io.atmosphere import AtmosphereModel
from ..io.lines.atomic import LineCatalog


def compute_transp(
    catalog: LineCatalog,
    populations,  # unused: TXNXN and Boltzmann factors are computed on the device
    atmosphere: AtmosphereModel,
    cutoff: float = 1e-3,
    continuum_absorption: Optional[np.ndarray] = None,
    wavelength_grid: Optional[np.ndarray] = None,
    continuum_absorption_full: Optional[np.ndarray] = None,
    wavelength_grid_full: Optional[np.ndarray] = None,
    microturb_kms: float = 0.0,
    device="cuda",
) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Line-centre opacity TRANSP[n_lines, L], valid mask and centre bins."""
    if continuum_absorption is None or wavelength_grid is None:
        raise ValueError(
            "compute_transp needs continuum_absorption and wavelength_grid: KAPMIN is the "
            "continuum at each line centre times the cutoff, with nothing to fall back on"
        )
    if continuum_absorption_full is not None or wavelength_grid_full is not None:
        raise NotImplementedError("full-range KAPMIN tables are not used on the default path")
    lib = _native.load()
    dcat = DeviceCatalog(catalog, device)
    datm = DeviceAtmosphere(atmosphere, device)
    dgrid = DeviceGrid(wavelength_grid, device=device)
    L = atmosphere.layers
    n = dcat.n_lines
    kap = torch.from_numpy(np.ascontiguousarray(continuum_absorption, np.float64)).to(dgrid.wavelength.device)
    tr = torch.zeros((max(n, 1), L), dtype=torch.float64, device=kap.device)
    va = torch.zeros((max(n, 1), L), dtype=torch.uint8, device=kap.device)
    ce = torch.zeros(max(n, 1), dtype=torch.int32, device=kap.device)
    opt = make_options(cutoff=cutoff, microturb_kms=microturb_kms, precision="fp64")
    _native.check(lib.ks_transp(C.byref(dcat.rec), C.byref(datm.rec), C.byref(dgrid.rec), C.byref(opt),
                                C.c_void_p(kap.data_ptr()), C.c_void_p(tr.data_ptr()),
                                C.c_void_p(va.data_ptr()), C.c_void_p(ce.data_ptr()), stream_handle()))
    torch.cuda.synchronize()
    tr_h = dcat.to_catalog_order(tr[:n].cpu().numpy())
    va_h = dcat.to_catalog_order(va[:n].cpu().numpy().astype(bool))
    ce_h = dcat.to_catalog_order(ce[:n].cpu().numpy().astype(np.int64))
    return tr_h, va_h, ce_h


def compute_asynth_from_transp(
    transp: np.ndarray,
    catalog: LineCatalog,
    atmosphere: AtmosphereModel,
    wavelength_grid: np.ndarray,
    valid_mask: Optional[np.ndarray] = None,
    populations=None,
    cutoff: float = 1e-3,
    continuum_absorption: Optional[np.ndarray] = None,
    continuum_absorption_full: Optional[np.ndarray] = None,
    wavelength_grid_full: Optional[np.ndarray] = None,
    metal_tables=None,
    grid_origin: Optional[float] = None,
    device="cuda",
    stats: Optional[dict] = None,
) -> np.ndarray:
    """ASYNTH[L, n]: centre + Voigt/far-wing accumulation, times STIM (FP64)."""
    lib = _native.load()
    dcat = DeviceCatalog(catalog, device)
    datm = DeviceAtmosphere(atmosphere, device)
    dgrid = DeviceGrid(wavelength_grid, grid_origin=grid_origin, device=device)
    L = atmosphere.layers
    n = dcat.n_lines
    dev = dgrid.wavelength.device
    order = dcat.order
    tr = np.ascontiguousarray(transp, np.float64)
    va = np.ones_like(tr, dtype=np.uint8) if valid_mask is None else np.ascontiguousarray(valid_mask, np.uint8)
    if order is not None:
        tr, va = tr[order], va[order]
    tr_d = torch.from_numpy(np.ascontiguousarray(tr)).to(dev)
    va_d = torch.from_numpy(np.ascontiguousarray(va)).to(dev)
    if continuum_absorption is None or continuum_absorption.shape != (L, dgrid.n):
        kap = torch.zeros((L, dgrid.n), dtype=torch.float64, device=dev)
    else:
        kap = torch.from_numpy(np.ascontiguousarray(continuum_absorption, np.float64)).to(dev)
    opt = make_options(cutoff=cutoff, precision="fp64")
    ws = C.c_size_t()
    _native.check(lib.ks_workspace_size(n, L, dgrid.n, C.byref(opt), C.byref(ws)))
    work = torch.empty(int(ws.value), dtype=torch.uint8, device=dev)
    out = torch.empty((L, dgrid.n), dtype=torch.float64, device=dev)
    st = _native.KsStats()
    _native.check(lib.ks_asynth(C.byref(dcat.rec), C.byref(datm.rec), C.byref(dgrid.rec), C.byref(opt),
                                C.c_void_p(tr_d.data_ptr()), C.c_void_p(va_d.data_ptr()),
                                C.c_void_p(kap.data_ptr()), C.c_void_p(work.data_ptr()), int(ws.value),
                                C.c_void_p(out.data_ptr()), C.byref(st), stream_handle()))
    torch.cuda.synchronize()
    if stats is not None:
        stats.update(st.as_dict())
    return out.cpu().numpy()
