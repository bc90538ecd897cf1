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

:class:`AtmosphereDiffSynthesizer` takes its atmosphere from an ATLAS ``.atm``
model through the FP64 population stage on the GPU (``ks_populations``) and
adds gradients with respect to the log10 abundances of chosen elements: the
adjoint's atmosphere terms (``ks_synthesize_adjoint_atmos``: dLoss/d ln
population per species and depth, d ln mass density, dXNE, dTXNXN) contracted
with the forward-mode derivatives of the population stage
(``ks_populations_tangent``).  The continuum opacity tables come from the
converted model and are held fixed.
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
from .physics.populations import DevicePopulations, PopulationTangents

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

    def forward(self, d_gf=None, d_gr=None, d_gs=None, d_gw=None, stats: bool = False):
        """(F_total, F_cont) at the given offsets; with ``stats`` the call's counters
        (valid pairs and evaluations: a change between two runs means a TRANSP gate or
        a wing reach step was crossed) are left in :attr:`last_stats`."""
        self.set_offsets(d_gf, d_gr, d_gs, d_gw)
        st = _native.KsStats() if stats else None
        _native.check(self.lib.ks_synthesize(
            C.byref(self.cat.rec), C.byref(self.atm.rec), C.byref(self.grid.rec), C.byref(self.opt),
            _ptr(self.ws), self.ws.numel(), _ptr(self.flux_total), _ptr(self.flux_cont), None,
            C.byref(st) if st is not None else None, None))
        if st is not None:
            self.last_stats = st.as_dict()
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


class AtmosphereDiffSynthesizer(DiffSynthesizer):
    """A :class:`DiffSynthesizer` whose atmosphere is recomputed from an ``.atm``
    model on the GPU for every evaluation, with gradients also for the log10
    abundances of ``elements`` (atomic numbers).  ``continuum``: the converted
    model of the same atmosphere, for its continuum coefficient tables."""

    POP_FIELDS = ("electron_density", "mass_density", "xnf_h", "xnf_he1", "xnf_h2")

    def __init__(self, catalog: LineCatalog, atm_model, continuum: AtmosphereModel, wavelength: np.ndarray,
                 elements, device="cuda"):
        self.pops = DevicePopulations([atm_model], device=device).run()
        super().__init__(catalog, self.pops.atmosphere(0, continuum), wavelength, device)
        self.elements = [int(z) for z in elements]
        self.xabund0 = self.pops.inputs[0]["xabund"].clone()
        self.tangents = PopulationTangents(self.pops, 0, self.elements)
        dev = self.ws.device
        L = self.atm.n_layers
        # lines grouped by species (each group in row order) for the adjoint's atmosphere sums
        e = np.asarray(catalog.element_idx, dtype=np.int64)
        ion = np.asarray(catalog.ion_stages, dtype=np.int64)
        n_ion, n_elem = int(self.atm.rec.n_ion), int(self.atm.rec.n_elem)
        ok = (e >= 0) & (e < n_elem) & (ion >= 1) & (ion <= n_ion)
        species = np.where(ok, (ion - 1) * n_elem + e, -1)
        rows = np.nonzero(ok)[0]
        order = rows[np.argsort(species[rows], kind="stable")]
        grp, first = np.unique(species[order], return_index=True)
        first = np.append(first, order.size)
        self._order = torch.from_numpy(order.astype(np.int32)).to(dev)
        self._first = torch.from_numpy(first.astype(np.int32)).to(dev)
        self._species = torch.from_numpy(grp.astype(np.int32)).to(dev)
        self.g_lnpop = torch.empty((L, n_ion, n_elem), dtype=torch.float64, device=dev)
        self.g_lnrho = torch.empty(L, dtype=torch.float64, device=dev)
        self.g_xne = torch.empty(L, dtype=torch.float64, device=dev)
        self.g_txnxn = torch.empty(L, dtype=torch.float64, device=dev)
        rec = _native.KsAtmGrad()
        rec.line_order = self._order.data_ptr()
        rec.group_first = self._first.data_ptr()
        rec.group_species = self._species.data_ptr()
        rec.n_groups = int(grp.size)
        rec.d_ln_population = self.g_lnpop.data_ptr()
        rec.d_ln_mass_density = self.g_lnrho.data_ptr()
        rec.d_electron_density = self.g_xne.data_ptr()
        rec.d_txnxn = self.g_txnxn.data_ptr()
        self.grad_rec = rec

    def set_abundances(self, d_ab=None):
        """Scale the selected elements' abundances by 10**d_ab (dex, device tensor
        [n_elements] or None) and recompute the populations into the synthesis
        atmosphere."""
        key = None if d_ab is None else d_ab.detach().to(torch.float64).clone()
        last = getattr(self, "_last_ab", ())
        if last != () and ((key is None and last is None) or
                           (key is not None and last is not None and torch.equal(key, last))):
            return  # the populations of these abundances are already in the atmosphere
        self._last_ab = key
        xab = self.xabund0.clone()
        if d_ab is not None:
            idx = torch.tensor([z - 1 for z in self.elements], dtype=torch.long, device=xab.device)
            xab[idx] = xab[idx] * torch.pow(torch.tensor(10.0, dtype=torch.float64, device=xab.device),
                                            d_ab.to(torch.float64))
        self.pops.inputs[0]["xabund"].copy_(xab)
        self.pops.run()
        out = self.pops.outputs[0]
        for f in self.POP_FIELDS:
            self.atm.t[f].copy_(out[f])
        self.atm.t["population"].copy_(out["population_per_ion"])

    def forward(self, d_gf=None, d_gr=None, d_gs=None, d_gw=None, d_ab=None, stats: bool = False):
        self.set_abundances(d_ab)
        return super().forward(d_gf, d_gr, d_gs, d_gw, stats=stats)

    def adjoint(self, g_flux_total: torch.Tensor, d_gf=None, d_gr=None, d_gs=None, d_gw=None, d_ab=None):
        """Line-parameter gradients as :meth:`DiffSynthesizer.adjoint`, then
        dLoss/dlog10 XABUND of each selected element."""
        self.set_abundances(d_ab)
        self.set_offsets(d_gf, d_gr, d_gs, d_gw)
        g = g_flux_total.to(torch.float64).contiguous()
        st = _native.KsStats()
        _native.check(self.lib.ks_synthesize_adjoint_atmos(
            C.byref(self.cat.rec), C.byref(self.atm.rec), C.byref(self.grid.rec), C.byref(self.opt),
            _ptr(self.ws), self.ws.numel(), _ptr(g), _ptr(self.flux_total), _ptr(self.flux_cont),
            _ptr(self.grads[0]), _ptr(self.grads[1]), _ptr(self.grads[2]), _ptr(self.grads[3]),
            C.byref(self.grad_rec), C.byref(st), None))
        self.skipped = int(st.maxj_wavelengths)
        self.tangents.run()
        return tuple(t.clone() for t in self.grads) + (self.abundance_gradient(),)

    def abundance_gradient(self) -> torch.Tensor:
        """Contract the adjoint's atmosphere terms with the population tangents:
        dL/dθ = sum_d [ sum_s g_lnpop dPOP/POP + g_lnrho dRHO/RHO + g_xne dXNE
        + g_txnxn dTXNXN ], TXNXN = (XNF_H + 0.42 XNF_HE1 + 0.85 XNF_H2)
        (max(T, 1) / 10^4)^0.3 as the per-depth state forms it."""
        out = self.pops.outputs[0]
        dd = self.tangents.d
        pop = out["population_per_ion"]
        # only species with lines carry a gradient; the rest (and empty ions) are left out
        use = (self.g_lnpop != 0) & (pop != 0)
        w = torch.where(use, self.g_lnpop / torch.where(use, pop, torch.ones_like(pop)), torch.zeros_like(pop))
        t_pop = torch.einsum("lis,elis->e", w, dd["population_per_ion"])
        t_rho = torch.einsum("l,el->e", self.g_lnrho / out["mass_density"], dd["mass_density"])
        t_xne = torch.einsum("l,el->e", self.g_xne, dd["electron_density"])
        temp = torch.clamp(self.pops.inputs[0]["temperature"], min=1.0)
        fac = torch.pow(temp / 10000.0, 0.3)
        dtx = (dd["xnf_h"] + 0.42 * dd["xnf_he1"] + 0.85 * dd["xnf_h2"]) * fac[None, :]
        t_tx = torch.einsum("l,el->e", self.g_txnxn, dtx)
        return t_pop + t_rho + t_xne + t_tx


class AtmosphereSynthesisFunction(torch.autograd.Function):
    """(line offsets x4, abundance offsets [n_elements]) -> (F_total, F_cont)."""

    @staticmethod
    def forward(ctx, ds: AtmosphereDiffSynthesizer, d_gf, d_gr, d_gs, d_gw, d_ab):
        ft, fc = ds.forward(d_gf, d_gr, d_gs, d_gw, d_ab)
        ctx.ds = ds
        ctx.save_for_backward(d_gf, d_gr, d_gs, d_gw, d_ab)
        ft, fc = ft.clone(), fc.clone()
        ctx.mark_non_differentiable(fc)
        return ft, fc

    @staticmethod
    def backward(ctx, g_ft, g_fc):
        d_gf, d_gr, d_gs, d_gw, d_ab = ctx.saved_tensors
        grads = ctx.ds.adjoint(g_ft, d_gf, d_gr, d_gs, d_gw, d_ab)
        return (None,) + tuple(grads)


def synthesize_atmosphere(ds: AtmosphereDiffSynthesizer, d_gf, d_gr, d_gs, d_gw, d_ab):
    """Differentiable (F_total, F_cont) in the line offsets and the abundance offsets."""
    return AtmosphereSynthesisFunction.apply(ds, d_gf, d_gr, d_gs, d_gw, d_ab)
