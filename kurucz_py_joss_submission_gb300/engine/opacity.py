"""Synthesis driver with the reference's stage order, on the GPU.

``run_synthesis`` replaces synthe_py/engine/opacity.py:2084 for the plain-
line LTE path: atmosphere (.npz) load, grid (:2143), catalog with the DELLIM
window (:2175), then the fused device synthesis -- continuum (:2236),
TRANSP (:2320), ASYNTH (:2352), SLINEC source (:3619, :3678) and the JOSH
transfer (:3788) -- the F_nu -> F_lambda conversion (:3855-3861) and the
``.spec`` writer (:3891).  ``SYNTHE_PY_STAGE_DUMPS`` writes the same stage
files as the reference (stage_3_transp, stage_4_asynth, stage_5_rt).
"""

from __future__ import annotations

import logging
import math
import os
import time
from pathlib import Path
from typing import Dict

import numpy as np
import torch

from .. import _native
from ..config import SynthesisConfig
from ..device import DeviceAtmosphere, DeviceCatalog, DeviceGrid, Synthesizer, make_options
from ..io import atmosphere as atm_io
from ..io import export
from ..io.lines import atomic
from .buffers import SynthResult

logger = logging.getLogger(__name__)

C_LIGHT_NM_PER_S = 2.99792458e17


def flux_nu_to_lambda(wavelength: np.ndarray, flux_hz: np.ndarray) -> np.ndarray:
    """F_lambda = F_nu * c / lambda^2 with c in nm/s (opacity.py:3855-3861)."""
    return flux_hz * (C_LIGHT_NM_PER_S / np.maximum(wavelength ** 2, 1e-40))


def _build_wavelength_grid(cfg: SynthesisConfig) -> np.ndarray:
    """Geometric grid of opacity.py:526 (native: sequential multiplication)."""
    g = cfg.wavelength_grid
    if g.resolution <= 0.0:
        raise ValueError("the log-lambda grid needs a resolving power above zero")
    L = _native.load()
    n = L.ks_wavelength_grid(g.start, g.end, g.resolution, None, 0)
    if n < 0:
        raise ValueError(L.ks_last_error().decode())
    out = np.zeros(n)
    L.ks_wavelength_grid(g.start, g.end, g.resolution, out.ctypes.data_as(_native.PD), n)
    return out


def _nearest_grid_indices(grid: np.ndarray, values: np.ndarray) -> np.ndarray:
    """Centre bins of opacity.py:550 computed by the device kernel."""
    import ctypes as C

    L = _native.load()
    dgrid = DeviceGrid(grid)
    v = torch.from_numpy(np.ascontiguousarray(values, np.float64)).to(dgrid.wavelength.device)
    out = torch.empty(max(v.numel(), 1), dtype=torch.int32, device=v.device)
    _native.check(L.ks_line_bins(C.byref(dgrid.rec), C.c_void_p(v.data_ptr()), v.numel(),
                                 C.c_void_p(out.data_ptr()), None,
                                 C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    return out[: v.numel()].cpu().numpy().astype(np.int64)


def _load_atmosphere(cfg: SynthesisConfig) -> atm_io.AtmosphereModel:
    path = cfg.atmosphere.npz_path or cfg.atmosphere.model_path
    path = Path(path)
    if path.suffix != ".npz":
        cand = path.with_suffix(".npz")
        if not cand.exists():
            raise FileNotFoundError(
                f"Could not find cached .npz atmosphere file for {path}; convert it first "
                "(synthe_py/tools/convert_atm_to_npz.py) or pass --npz")
        path = cand
    atm = atm_io.load_cached(path)
    if cfg.populations == "gpu":
        from ..physics.populations import DevicePopulations

        model = Path(cfg.atmosphere.model_path)
        if model.suffix == ".npz":
            raise ValueError("--populations gpu needs the ATLAS .atm model as MODEL")
        atm = DevicePopulations([model]).run().atmosphere(0, continuum=atm)
    return atm


def run_synthesis(cfg: SynthesisConfig) -> SynthResult:
    t0 = time.perf_counter()
    timings: Dict[str, float] = {}
    atm = _load_atmosphere(cfg)
    timings["atmosphere load"] = time.perf_counter() - t0

    t = time.perf_counter()
    wavelength_full = _build_wavelength_grid(cfg)
    grid_origin = float(wavelength_full[0]) if wavelength_full.size else None
    wavelength = wavelength_full[:: cfg.wavelength_subsample] if cfg.wavelength_subsample > 1 else wavelength_full
    timings["wavelength grid"] = time.perf_counter() - t

    t = time.perf_counter()
    g = cfg.wavelength_grid
    if cfg.line_filter:
        catalog = atomic.load_catalog_window(cfg.line_data.atomic_catalog, g.start, g.end, sort=True)
    else:
        catalog = atomic.load_catalog(cfg.line_data.atomic_catalog)
    timings["line catalog"] = time.perf_counter() - t
    logger.info("Catalog: %d lines, grid: %d points", len(catalog), wavelength.size)

    t = time.perf_counter()
    dcat = DeviceCatalog(catalog, hydrogen=not cfg.skip_hydrogen_wings, helium=cfg.enable_helium_wings)
    datm = DeviceAtmosphere(atm)
    dgrid = DeviceGrid(wavelength, grid_origin=grid_origin)
    opt = make_options(cutoff=cfg.cutoff, microturb_kms=g.velocity_microturb, rhoxj=cfg.rhoxj_scale,
                       precision=cfg.precision, tile_bins=cfg.tile_bins,
                       warps_per_tile=cfg.warps_per_tile)
    syn = Synthesizer(dcat, datm, dgrid, opt, keep_asynth=True)
    stats = syn.run(stats=True)
    torch.cuda.synchronize()
    timings["synthesis (GPU)"] = time.perf_counter() - t

    flux_total_hz = syn.flux_total.cpu().numpy()
    flux_cont_hz = syn.flux_cont.cpu().numpy()
    flux_total = flux_nu_to_lambda(wavelength, flux_total_hz)
    flux_cont = flux_nu_to_lambda(wavelength, flux_cont_hz)

    dump_dir = os.environ.get("SYNTHE_PY_STAGE_DUMPS")
    if dump_dir:
        _stage_dumps(Path(dump_dir), cfg, catalog, atm, wavelength, syn, flux_total_hz, flux_cont_hz)

    timings["total pipeline"] = time.perf_counter() - t0
    for k, v in timings.items():
        logger.info("Timing: %s in %.3fs", k, v)
    result = SynthResult(wavelength=wavelength.copy(), intensity=flux_total, continuum=flux_cont,
                         timings=timings, stats=stats)
    if cfg.output.spec_path is not None:
        export.write_spec_file(result, cfg.output.spec_path)
    if cfg.output.diagnostics_path is not None:
        Path(cfg.output.diagnostics_path).parent.mkdir(parents=True, exist_ok=True)
        np.savez(cfg.output.diagnostics_path, wavelength=wavelength,
                 line_opacity=syn.asynth.double().cpu().numpy(), flux_total=flux_total,
                 flux_continuum=flux_cont)
    return result


def _stage_dumps(path: Path, cfg, catalog, atm, wavelength, syn, ft_hz, fc_hz) -> None:
    """Stage files in the reference's layout (opacity.py:2333-2405, :3803-3815)."""
    from ..physics.line_opacity import compute_transp
    from .continuum import build_depth_continuum

    path.mkdir(parents=True, exist_ok=True)
    ca, cs = build_depth_continuum(atm, wavelength)
    transp, valid, cidx = compute_transp(catalog, None, atm, cfg.cutoff, ca + cs, wavelength,
                                         microturb_kms=cfg.wavelength_grid.velocity_microturb)
    order = np.argsort(catalog.catalog_index)
    np.savez(path / "stage_3_transp.npz", transp=transp[order], valid_mask=valid[order],
             line_indices=cidx[order])
    full = syn.asynth.double().cpu().numpy()
    stage4 = full
    rec = syn.catalog.rec
    if rec.n_hydrogen or rec.n_helium:
        # the reference's stage-4 ASYNTH precedes the hydrogen profiles and
        # the helium wings (opacity.py:2395-2404, :2465, :3650): rerun without them
        nh, nhe = rec.n_hydrogen, rec.n_helium
        rec.n_hydrogen = rec.n_helium = 0
        try:
            syn.run()
            stage4 = syn.asynth.double().cpu().numpy()
        finally:
            rec.n_hydrogen, rec.n_helium = nh, nhe
    np.savez(path / "stage_4_asynth.npz", asynth=stage4, wavelength=wavelength)
    # the transfer's line opacity: absorption ASYNTH (1 - FSCAT), scattering
    # ASYNTH FSCAT (opacity.py:2416-2440, :3650-3661)
    rhox = np.asarray(atm.depth, dtype=np.float64)
    fscat = np.exp(-rhox / cfg.rhoxj_scale) if cfg.rhoxj_scale > 0.0 else np.zeros_like(rhox)
    np.savez(path / "stage_5_rt.npz", wavelength=wavelength, flux_total_hz=ft_hz, flux_cont_hz=fc_hz,
             flux_total=ft_hz, flux_cont=fc_hz, cont_abs=ca, cont_scat=cs,
             line_opacity=full * (1.0 - fscat[:, None]), line_scattering=full * fscat[:, None])
