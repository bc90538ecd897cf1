"""Differentiable synthesis: gradients of a spectrum loss with respect to the
line parameters, from hand-written adjoint kernels.

The parameters are offsets, in dex, of every line's log10 gf and log10
damping constants (radiative, Stark, van der Waals) from the catalog's
values: the catalog columns the synthesis reads (``gf``, ``cgf``,
``gamma_*``; synthe_py/io/lines/atomic.py:299-611 derives them from the gfall
logs) are scaled by 10**offset.  :class:`DiffSynthesizer` runs the FP64 fused
synthesis with the JOSH system solved to 1e-13 (``ks_synthesize``,
``exact_sweeps``) and its adjoint (``ks_synthesize_adjoint``);
:class:`SynthesisFunction` wraps both as a ``torch.autograd.Function`` so a
loss written in torch on the normalised flux back-propagates into the four
per-line offset tensors.

The TRANSP gates and the wing reach are step functions of the parameters and
are held fixed by the adjoint; wavelengths in the MAXJ = 1 branch contribute
no gradient (counted in :attr:`DiffSynthesizer.skipped`).
"""

from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np
import torch

from . import _native
from .device import DeviceAtmosphere, DeviceCatalog, DeviceGrid, _ptr, make_options
from .io.atmosphere import AtmosphereModel
from .io.lines.atomic import LineCatalog

PARAMS = ("gf", "gamma_rad", "gamma_stark", "gamma_vdw")


class DiffSynthesizer:
    """One atmosphere, one grid, one (wavelength-sorted) line list."""

    def __init__(self, catalog: LineCatalog, atm: AtmosphereModel, wavelength: np.ndarray, device="cuda"):
        self.lib = _native.load()
        self.cat = DeviceCatalog(catalog, device)
        if self.cat.order is not None:
            raise ValueError("DiffSynthesizer: give the catalog sorted by wavelength")
        self.atm = DeviceAtmosphere(atm, device)
        self.grid = DeviceGrid(wavelength, device=device)
        self.opt = make_options(precision="fp64", exact_sweeps=1)
        dev = self.grid.wavelength.device
        ws = C.c_size_t()
        _native.check(self.lib.ks_workspace_size(self.cat.n_lines, self.atm.n_layers, self.grid.n,
                                                 C.byref(self.opt), C.byref(ws)))
        self.ws = torch.empty(int(ws.value), dtype=torch.uint8, device=dev)
        self.base = {k: self.cat.t[k].clone() for k in ("gf", "cgf", "gamma_rad", "gamma_stark", "gamma_vdw")}
        n = self.grid.n
        self.flux_total = torch.empty(n, dtype=torch.float64, device=dev)
        self.flux_cont = torch.empty(n, dtype=torch.float64, device=dev)
        self.grads = [torch.empty(self.cat.n_lines, dtype=torch.float64, device=dev) for _ in PARAMS]
        self.skipped = 0

    def set_offsets(self, d_gf, d_gr, d_gs, d_gw):
        """Scale the device columns by 10**offset (offsets: device tensors [n_lines] or None)."""
        ten = torch.tensor(10.0, dtype=torch.float64, device=self.ws.device)
        for col, d in (("gf", d_gf), ("cgf", d_gf), ("gamma_rad", d_gr), ("gamma_stark", d_gs),
                       ("gamma_vdw", d_gw)):
            if d is None:
                self.cat.t[col].copy_(self.base[col])
            else:
                torch.mul(self.base[col], torch.pow(ten, d.to(torch.float64)), out=self.cat.t[col])

    def forward(self, d_gf=None, d_gr=None, d_gs=None, d_gw=None):
        self.set_offsets(d_gf, d_gr, d_gs, d_gw)
        _native.check(self.lib.ks_synthesize(
            C.byref(self.cat.rec), C.byref(self.atm.rec), C.byref(self.grid.rec), C.byref(self.opt),
            _ptr(self.ws), self.ws.numel(), _ptr(self.flux_total), _ptr(self.flux_cont), None, None, None))
        return self.flux_total, self.flux_cont

    def adjoint(self, g_flux_total: torch.Tensor, d_gf=None, d_gr=None, d_gs=None, d_gw=None):
        """Gradients (log10 gf, log10 gamma_rad, log10 gamma_stark, log10 gamma_vdw) for
        dLoss/dF_total = g_flux_total, at the given offsets."""
        self.set_offsets(d_gf, d_gr, d_gs, d_gw)
        g = g_flux_total.to(torch.float64).contiguous()
        st = _native.KsStats()
        _native.check(self.lib.ks_synthesize_adjoint(
            C.byref(self.cat.rec), C.byref(self.atm.rec), C.byref(self.grid.rec), C.byref(self.opt),
            _ptr(self.ws), self.ws.numel(), _ptr(g), _ptr(self.flux_total), _ptr(self.flux_cont),
            _ptr(self.grads[0]), _ptr(self.grads[1]), _ptr(self.grads[2]), _ptr(self.grads[3]),
            C.byref(st), None))
        self.skipped = int(st.maxj_wavelengths)
        return tuple(t.clone() for t in self.grads)


class SynthesisFunction(torch.autograd.Function):
    """(d_log_gf, d_log_gamma_rad, d_log_gamma_stark, d_log_gamma_vdw) ->
    (F_total, F_cont), F_nu per grid point; F_cont does not depend on the lines."""

    @staticmethod
    def forward(ctx, ds: DiffSynthesizer, d_gf, d_gr, d_gs, d_gw):
        ft, fc = ds.forward(d_gf, d_gr, d_gs, d_gw)
        ctx.ds = ds
        ctx.save_for_backward(d_gf, d_gr, d_gs, d_gw)
        ft, fc = ft.clone(), fc.clone()
        ctx.mark_non_differentiable(fc)
        return ft, fc

    @staticmethod
    def backward(ctx, g_ft, g_fc):
        d_gf, d_gr, d_gs, d_gw = ctx.saved_tensors
        grads = ctx.ds.adjoint(g_ft, d_gf, d_gr, d_gs, d_gw)
        return (None,) + tuple(grads)


def synthesize(ds: DiffSynthesizer, d_gf, d_gr, d_gs, d_gw):
    """Differentiable (F_total, F_cont)."""
    return SynthesisFunction.apply(ds, d_gf, d_gr, d_gs, d_gw)
