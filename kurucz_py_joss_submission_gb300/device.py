"""Device-resident inputs and the fused synthesis plan.

``DeviceAtmosphere``, ``DeviceGrid`` and ``DeviceCatalog`` hold the inputs in
HBM (torch tensors own the memory) and expose the C-ABI records that point
at them.  ``Synthesizer`` sizes one workspace for a (catalog, atmosphere,
grid) triple and runs ``ks_synthesize`` on the current CUDA stream, so a
synthesis is one call with no allocation once the plan exists.
"""

from __future__ import annotations

import ctypes as C
import warnings
from dataclasses import dataclass
from typing import Dict, Optional

import numpy as np
import torch

from . import _native
from .io.atmosphere import AtmosphereModel
from .io.lines.atomic import LineCatalog

PRECISIONS = {"mixed": _native.KS_PREC_MIXED, "fp64": _native.KS_PREC_FP64}


def _require_cuda(device) -> torch.device:
    dev = torch.device(device)
    if dev.type != "cuda":
        raise RuntimeError("the synthesis kernels run on a CUDA device only (no CPU fallback)")
    if not torch.cuda.is_available():
        raise RuntimeError("CUDA is not available: the GB300 synthesis path needs a GPU")
    return dev


def _dev(a: np.ndarray, dtype, device) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).to(device, non_blocking=False)


def _ptr(t: Optional[torch.Tensor]):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def stream_handle(stream: Optional[torch.cuda.Stream] = None) -> C.c_void_p:
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


class DeviceAtmosphere:
    """One converted atmosphere in HBM."""

    def __init__(self, atm: AtmosphereModel, device="cuda"):
        dev = _require_cuda(device)
        L = atm.layers
        f64 = np.float64
        self.n_layers = L
        self.t: Dict[str, torch.Tensor] = {}

        def put(name, arr):
            if arr is None:
                return None
            self.t[name] = _dev(arr, f64, dev)
            return self.t[name]

        put("rhox", atm.depth)
        put("temperature", atm.temperature)
        put("electron_density", atm.electron_density)
        put("mass_density", atm.mass_density)
        put("hckt", atm.hckt)
        put("xnf_h", atm.xnf_h)
        put("xnf_he1", atm.xnf_he1)
        put("xnf_h2", atm.xnf_h2)
        pop = atm.population_per_ion if atm.population_per_ion is not None else np.zeros((L, 1, 1))
        dop = atm.doppler_per_ion if atm.doppler_per_ion is not None else np.zeros((L, 1, 1))
        put("population", pop)
        put("doppler", dop)
        put("wledge", atm.continuum_wledge)
        put("half_edge", atm.continuum_half_edge)
        put("delta_edge", atm.continuum_delta_edge)
        put("cont_abs_coeff", atm.continuum_abs_coeff)
        put("cont_scat_coeff", atm.continuum_scat_coeff)
        put("turbulent_velocity", atm.turbulent_velocity)
        rec = _native.KsAtmos()
        rec.n_layers = L
        for name in ("rhox", "temperature", "electron_density", "mass_density", "hckt", "xnf_h",
                     "xnf_he1", "xnf_h2", "population", "doppler", "wledge", "half_edge",
                     "delta_edge", "cont_abs_coeff", "cont_scat_coeff", "turbulent_velocity"):
            t = self.t.get(name)
            setattr(rec, name, t.data_ptr() if t is not None else None)
        rec.n_ion = int(pop.shape[1])
        rec.n_elem = int(pop.shape[2])
        rec.n_edge = int(atm.continuum_wledge.size) if atm.continuum_wledge is not None else 0
        rec.coeff_log10 = 1 if atm.continuum_coeff_log10 else 0
        self.rec = rec


class DeviceGrid:
    """The log-lambda grid in HBM."""

    def __init__(self, wavelength: np.ndarray, grid_origin: Optional[float] = None, device="cuda"):
        dev = _require_cuda(device)
        self.wavelength_host = np.ascontiguousarray(wavelength, dtype=np.float64)
        self.wavelength = _dev(self.wavelength_host, np.float64, dev)
        self.n = int(self.wavelength_host.size)
        rec = _native.KsGrid()
        rec.n = self.n
        rec.wavelength = self.wavelength.data_ptr()
        rec.grid_origin = float(grid_origin if grid_origin is not None else
                                (self.wavelength_host[0] if self.n else 0.0))
        self.rec = rec


# fort.19's CODEX species (io/lines/fort19.py:21-24): the ions with
# continuum-merge limits
FORT19_CODEX = np.array([1.0, 2.0, 2.01, 6.0, 6.01, 12.0, 12.01, 13.0, 13.01, 14.0, 14.01, 20.0, 20.01, 8.0,
                         11.0, 5.0, 19.0])


def inv_order(order: np.ndarray) -> np.ndarray:
    """Catalog row -> device row, for a device order given as catalog rows."""
    inv = np.empty_like(order)
    inv[order] = np.arange(order.size)
    return inv


class DeviceCatalog:
    """A line catalog in HBM, sorted by wavelength (the kernels require it).

    ``order`` maps device rows to catalog rows, for returning per-line
    results in catalog order."""

    COLUMNS_F64 = ("wavelength", "gf", "cgf", "gamma_rad", "gamma_stark", "gamma_vdw",
                   "excitation_energy")
    COLUMNS_I32 = ("element_idx", "ion_stages", "line_types")
    COLUMNS_U8 = ("process_mask", "asynth_mask")

    def __init__(self, cat: LineCatalog, device="cuda", hydrogen: bool = True, helium: bool = True):
        """``hydrogen`` / ``helium``: add the hydrogen profiles and the helium
        wing pass (SynthesisConfig.skip_hydrogen_wings / enable_helium_wings,
        engine/opacity.py:2465, :2515); without them those lines keep only
        what TRANSP/ASYNTH give them."""
        dev = _require_cuda(device)
        if cat.is_sorted():
            self.order = None
            src = cat
        else:
            self.order = np.argsort(cat.wavelength, kind="stable")
            src = cat.take(self.order)
        self.n_lines = len(src)
        self.t: Dict[str, torch.Tensor] = {}
        for k in self.COLUMNS_F64:
            self.t[k] = _dev(getattr(src, k), np.float64, dev)
        for k in self.COLUMNS_I32:
            self.t[k] = _dev(getattr(src, k), np.int32, dev)
        for k in self.COLUMNS_U8:
            self.t[k] = _dev(getattr(src, k), np.uint8, dev)
        self.host = src
        rec = _native.KsLines()
        rec.n_lines = self.n_lines
        rec.wavelength = self.t["wavelength"].data_ptr()
        rec.gf = self.t["gf"].data_ptr()
        rec.cgf = self.t["cgf"].data_ptr()
        rec.gamma_rad = self.t["gamma_rad"].data_ptr()
        rec.gamma_stark = self.t["gamma_stark"].data_ptr()
        rec.gamma_vdw = self.t["gamma_vdw"].data_ptr()
        rec.elo_cm = self.t["excitation_energy"].data_ptr()
        rec.element_idx = self.t["element_idx"].data_ptr()
        rec.ion_stage = self.t["ion_stages"].data_ptr()
        rec.line_type = self.t["line_types"].data_ptr()
        rec.process_mask = self.t["process_mask"].data_ptr()
        rec.asynth_mask = self.t["asynth_mask"].data_ptr()
        rec.sorted_by_wavelength = 1
        # hydrogen lines (line types -1/-2, neutral H; engine/opacity.py:1773-1778):
        # their device rows listed in catalog order, the order the reference
        # adds their profiles in
        lt = np.asarray(cat.line_types)
        hyd = np.flatnonzero(((lt == -1) | (lt == -2)) & (np.asarray(cat.ion_stages) == 1) & hydrogen)
        self.n_hydrogen = int(hyd.size)
        if self.n_hydrogen > 65536:
            raise ValueError(f"{self.n_hydrogen} hydrogen lines: the synthesis takes at most 65536")
        if self.n_hydrogen:
            lo = np.asarray(cat.n_lower)[hyd]
            up = np.maximum(np.asarray(cat.n_upper)[hyd], lo + 1)
            if np.any(up + 2 > 96):
                raise ValueError("hydrogen line with an upper level above 94: the profile tables "
                                 "(ASUM) end at level 96")
            rows = hyd if self.order is None else inv_order(self.order)[hyd]
            self.t["hydrogen_rows"] = _dev(rows, np.int32, dev)
            self.t["hydrogen_n_lower"] = _dev(np.asarray(cat.n_lower)[hyd], np.int32, dev)
            self.t["hydrogen_n_upper"] = _dev(np.asarray(cat.n_upper)[hyd], np.int32, dev)
            rec.n_hydrogen = self.n_hydrogen
            rec.hydrogen_rows = self.t["hydrogen_rows"].data_ptr()
            rec.hydrogen_n_lower = self.t["hydrogen_n_lower"].data_ptr()
            rec.hydrogen_n_upper = self.t["hydrogen_n_upper"].data_ptr()
        # fort.19 lines (io/lines/fort19.py:343-347) other than hydrogen and
        # helium: the NORMAL ones (line type 0 with NBLO/NBUP set), the
        # autoionizing ones (TYPE 1) and the merged-continuum records get
        # _add_fort19_asynth's profiles (engine/opacity.py:1335-1541) here,
        # with the records' continuum-merge limits
        nb = np.abs(np.asarray(cat.n_lower)) + np.abs(np.asarray(cat.n_upper))
        # continuum-merge limits of fort.19 records (fort19.py:330-338): NCON
        # = ISO2 when ISO1 is 0, NELIONX = the species' CONTX column
        ncon = np.where((np.asarray(cat.iso1) == 0) & (np.asarray(cat.iso2) > 0), np.asarray(cat.iso2), 0)
        match = np.isclose(np.asarray(cat.code)[:, None], FORT19_CODEX[None, :], rtol=0.0, atol=1e-3)
        nelionx = np.where(match.any(axis=1), match.argmax(axis=1) + 1, 0)
        known = (np.asarray(cat.element_idx) >= 0) & (np.asarray(cat.ion_stages) >= 1)
        # merged-continuum records: LABELP CONTINUU makes the fort.19 type
        # NLAST = XJP (or NBUP) and gf x (2 XJ + 1) (fort19.py:304-307)
        clab = np.asarray(cat.continuum_label) != 0
        nlast = np.where(np.asarray(cat.xjp) > 0.0, np.asarray(cat.xjp).astype(np.int64),
                         np.asarray(cat.n_upper).astype(np.int64))
        cont = clab & (nlast > 3) & known
        normal = (lt == 0) & (nb != 0) & known & ~clab
        aut = (lt == 1) & known & ~clab
        f19 = np.flatnonzero(normal | aut | cont)
        odd = clab & ~cont & ((nlast == 1) | ((nlast <= 0) & (nb != 0)))
        self.n_fort19_skipped = int(np.count_nonzero(odd))
        if self.n_fort19_skipped:
            warnings.warn(f"{self.n_fort19_skipped} CONTINUU records of NLAST <= 1 contribute no opacity here",
                          RuntimeWarning, stacklevel=2)
        self.n_f19 = int(f19.size)
        if self.n_f19 > 65536:
            raise ValueError(f"{self.n_f19} fort.19 lines: the synthesis takes at most 65536")
        if self.n_f19:
            is_cont = cont[f19]
            is_aut = (lt[f19] == 1) & ~is_cont
            wl = np.asarray(cat.wavelength)[f19]
            gf = 10.0 ** np.asarray(cat.log_gf, dtype=np.float64)[f19]
            freq = 2.99792458e17 / np.maximum(wl, 1.0e-30)
            denom = 12.5664 * freq
            # the fort.19 record's single-precision fields (fort19.py:352-402):
            # NORMAL lines CGF and the normalised damping constants,
            # autoionizing lines gf and the damping constants of the gfall
            # logs (a positive GS encodes a negative ASHORE)
            f32 = lambda x: np.asarray(x, dtype=np.float32).astype(np.float64)  # noqa: E731
            grl, gsl, gwl = (np.asarray(getattr(cat, k))[f19] for k in
                             ("gamma_rad_log", "gamma_stark_log", "gamma_vdw_log"))
            g_r, g_s, g_w = (np.asarray(getattr(cat, k))[f19] for k in ("gamma_rad", "gamma_stark", "gamma_vdw"))
            with np.errstate(over="ignore"):
                aut_r = np.where(grl != 0.0, 10.0 ** grl, g_r * denom)
                aut_s = np.where(gsl > 0.0, -(10.0 ** (-gsl)), np.where(gsl < 0.0, 10.0 ** gsl, g_s * denom))
                aut_w = np.where(gwl != 0.0, 10.0 ** gwl, g_w * denom)
            code = np.asarray(cat.code)[f19]
            nelem = (code + 1e-6).astype(np.int64)
            icharge = ((code - nelem) * 100.0 + 0.1).astype(np.int64)
            nelion = nelem * 6 - 6 + (icharge + 1)
            nelion = np.where((nelem > 19) & (nelem < 29) & (icharge > 5),
                              6 * (nelem + icharge * 10 - 30) - 1, nelion)
            gf_cont = gf * (2.0 * np.asarray(cat.xj)[f19] + 1.0)
            vals = {
                "cgf": f32(np.where(is_cont, gf_cont, np.where(is_aut, gf, (0.026538 / 1.77245) * gf / freq))),
                "gamma_rad": f32(np.where(is_aut, aut_r, g_r)),
                "gamma_stark": f32(np.where(is_aut, aut_s, g_s)),
                "gamma_vdw": f32(np.where(is_aut, aut_w, g_w)),
            }
            self.t["f19_rows"] = _dev(f19 if self.order is None else inv_order(self.order)[f19], np.int32, dev)
            self.t["f19_kind"] = _dev(np.where(is_cont, 2, np.where(is_aut, 1, 0)), np.int32, dev)
            self.t["f19_nlast"] = _dev(nlast[f19], np.int32, dev)
            self.t["f19_nelion"] = _dev(nelion, np.int32, dev)
            self.t["f19_ncon"] = _dev(np.where(normal[f19], ncon[f19], 0), np.int32, dev)
            self.t["f19_nelionx"] = _dev(nelionx[f19], np.int32, dev)
            for k, v in vals.items():
                self.t["f19_" + k] = _dev(v, np.float64, dev)
            rec.n_f19 = self.n_f19
            for k in ("rows", "kind", "nlast", "nelion", "ncon", "nelionx", "cgf", "gamma_rad", "gamma_stark",
                      "gamma_vdw"):
                setattr(rec, "f19_" + k, self.t["f19_" + k].data_ptr())
        # helium lines (line types -3/-4/-6; engine/opacity.py:2531-2544): the
        # helium wing pass, device rows in catalog order
        he = np.flatnonzero(np.isin(lt, (-3, -4, -6)) & helium)
        self.n_helium = int(he.size)
        if self.n_helium > 65536:
            raise ValueError(f"{self.n_helium} helium lines: the synthesis takes at most 65536")
        if self.n_helium:
            self.t["helium_rows"] = _dev(he if self.order is None else inv_order(self.order)[he], np.int32, dev)
            # only fort.19 records (NBLO/NBUP set) carry the merge limits
            self.t["helium_ncon"] = _dev(np.where(nb[he] != 0, ncon[he], 0), np.int32, dev)
            self.t["helium_nelionx"] = _dev(nelionx[he], np.int32, dev)
            rec.n_helium = self.n_helium
            rec.helium_rows = self.t["helium_rows"].data_ptr()
            rec.helium_ncon = self.t["helium_ncon"].data_ptr()
            rec.helium_nelionx = self.t["helium_nelionx"].data_ptr()
        self.rec = rec

    def to_catalog_order(self, per_line: np.ndarray) -> np.ndarray:
        """Rows in device (sorted) order -> rows in catalog order."""
        if self.order is None:
            return per_line
        out = np.empty_like(per_line)
        out[self.order] = per_line
        return out


def check_flags(stream: Optional[torch.cuda.Stream] = None) -> None:
    """Synchronise the stream (default: the current one) and raise
    ``KsError`` (KS_ERR_DEVICE) if any synthesis on this device flagged an
    internal limit since the last check.  The calls themselves stay
    asynchronous; their flags are kept on the device until this is called."""
    s = stream if stream is not None else torch.cuda.current_stream()
    _native.check_device_flags(s.cuda_stream)


def make_options(cutoff=1e-3, microturb_kms=0.0, rhoxj=0.0, precision="mixed", tile_bins=0,
                 warps_per_tile=0, profile=False, short_class=0,
                 transfer_path=0, long_class=0, exact_sweeps=0) -> _native.KsOptions:
    opt = _native.KsOptions()
    opt.cutoff = float(cutoff)
    opt.microturb_kms = float(microturb_kms)
    opt.rhoxj = float(rhoxj)
    opt.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    opt.tile_bins = int(tile_bins)
    opt.warps_per_tile = int(warps_per_tile)
    opt.profile = 1 if profile else 0
    opt.short_class = int(short_class)
    opt.transfer_path = int(transfer_path)
    opt.long_class = int(long_class)
    opt.exact_sweeps = int(exact_sweeps)
    return opt


class Synthesizer:
    """Fused continuum -> TRANSP -> ASYNTH -> JOSH for one atmosphere.

    Owns the workspace and the outputs (``flux_total``/``flux_cont`` F_nu,
    ``asynth`` the line opacity).  ``run()`` enqueues the synthesis on the
    current stream and returns nothing; ``run(stats=True)`` synchronises and
    returns the counters."""

    def __init__(self, catalog: DeviceCatalog, atmosphere: DeviceAtmosphere, grid: DeviceGrid,
                 options: Optional[_native.KsOptions] = None, keep_asynth: bool = True):
        self.lib = _native.load()
        self.catalog, self.atmosphere, self.grid = catalog, atmosphere, grid
        self.options = options or make_options()
        dev = grid.wavelength.device
        ws = C.c_size_t()
        _native.check(self.lib.ks_workspace_size(catalog.n_lines, atmosphere.n_layers, grid.n,
                                                 C.byref(self.options), C.byref(ws)))
        self.workspace_bytes = int(ws.value)
        self.workspace = torch.empty(self.workspace_bytes, dtype=torch.uint8, device=dev)
        self.flux_total = torch.empty(grid.n, dtype=torch.float64, device=dev)
        self.flux_cont = torch.empty(grid.n, dtype=torch.float64, device=dev)
        fp64 = self.options.precision == _native.KS_PREC_FP64
        self.asynth = (torch.empty((atmosphere.n_layers, grid.n),
                                   dtype=torch.float64 if fp64 else torch.float32, device=dev)
                       if keep_asynth else None)

    def run(self, stats: bool = False, stream: Optional[torch.cuda.Stream] = None):
        st = _native.KsStats()
        status = self.lib.ks_synthesize(
            C.byref(self.catalog.rec), C.byref(self.atmosphere.rec), C.byref(self.grid.rec),
            C.byref(self.options), _ptr(self.workspace), self.workspace_bytes,
            _ptr(self.flux_total), _ptr(self.flux_cont), _ptr(self.asynth),
            C.byref(st) if stats else None, stream_handle(stream))
        _native.check(status)
        return st.as_dict() if stats else None

    def check(self, stream: Optional[torch.cuda.Stream] = None) -> None:
        """Raise if this or any earlier call on the device flagged an internal
        limit (see :func:`check_flags`)."""
        check_flags(stream)
