"""ctypes driver for the CPU oracle (``ks_oracle.c``) -- test infrastructure.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, always to verify results or as the timed CPU
reference, never as part of the product.

:func:`synthesize` follows the data flow of the reference driver
``synthe_py/engine/opacity.py:2084`` (``run_synthesis``) for the plain-line
LTE path: grid (``:2143``), centre bins (``:2201``), continuum (``:2236``),
TRANSP (``:2320``), ASYNTH (``:2352``), line source (``:3619``/``:3678``),
transfer (``:3788``) and the F_nu -> F_lambda conversion (``:3855-3861``).
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
import time
from pathlib import Path
from typing import Dict, Optional

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libks_oracle.so"
TABLES = HERE.parent / "kurucz_py_joss_submission_gb300" / "data" / "synthe_tables.npz"

_lib: Optional[C.CDLL] = None

P_D = C.POINTER(C.c_double)
P_I64 = C.POINTER(C.c_int64)
P_I32 = C.POINTER(C.c_int32)
P_U8 = C.POINTER(C.c_uint8)


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        L.kso_wavelength_grid.restype = C.c_int64
        L.kso_wavelength_grid.argtypes = [C.c_double, C.c_double, C.c_double, P_D, C.c_int64]
        L.kso_voigt.restype = C.c_double
        L.kso_voigt.argtypes = [C.c_double, C.c_double, P_D, P_D, P_D]
        L.kso_num_threads.restype = C.c_int
        _lib = L
    return _lib


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(t) if a is not None else None


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def set_threads(n: int) -> None:
    lib().kso_set_num_threads(int(n))


def set_exact_sweeps(on: bool) -> None:
    """Solve the JOSH system in FP64 to 1e-13 instead of the reference's FP32
    sweep (smooth fluxes, for differencing gradients); off = the reference."""
    lib().kso_set_exact_sweeps(1 if on else 0)


def num_threads() -> int:
    return int(lib().kso_num_threads())


def tables() -> Dict[str, np.ndarray]:
    with np.load(TABLES) as d:
        t = {k: np.asarray(d[k]) for k in d}
    L = lib()
    h0 = np.zeros(2001); h1 = np.zeros(2001); h2 = np.zeros(2001)
    L.kso_voigt_tables(_p(_d(t["tabvi"]), P_D), _p(_d(t["tabh1"]), P_D), C.c_int(t["tabvi"].size),
                       _p(h0, P_D), _p(h1, P_D), _p(h2, P_D))
    ex = np.zeros(1001); exf = np.zeros(1001)
    L.kso_exp_tables(_p(ex, P_D), _p(exf, P_D))
    t.update(h0tab=h0, h1tab=h1, h2tab=h2, extab=ex, extabf=exf)
    return t


def wavelength_grid(start: float, end: float, resolution: float) -> np.ndarray:
    L = lib()
    n = L.kso_wavelength_grid(start, end, resolution, None, 0)
    out = np.zeros(n)
    L.kso_wavelength_grid(start, end, resolution, _p(out, P_D), n)
    return out


def center_indices(grid: np.ndarray, wl: np.ndarray) -> np.ndarray:
    out = np.zeros(wl.size, dtype=np.int64)
    lib().kso_center_indices(_p(_d(grid), P_D), C.c_int64(grid.size), _p(_d(wl), P_D),
                             C.c_int64(wl.size), _p(out, P_I64))
    return out


def wing_indices(grid: np.ndarray, wl: np.ndarray, grid_origin: float) -> np.ndarray:
    out = np.zeros(wl.size, dtype=np.int64)
    lib().kso_wing_indices(_p(_d(grid), P_D), C.c_int64(grid.size), _p(_d(wl), P_D),
                           C.c_int64(wl.size), C.c_double(grid_origin), _p(out, P_I64))
    return out


def voigt(v: float, a: float, t: Dict[str, np.ndarray]) -> float:
    return lib().kso_voigt(v, a, _p(t["h0tab"], P_D), _p(t["h1tab"], P_D), _p(t["h2tab"], P_D))


def continuum(atm: Dict[str, np.ndarray], grid: np.ndarray):
    L = atm["temperature"].size
    n = grid.size
    wledge = _d(atm["wledge"])
    ca = np.zeros((L, n)); cs = np.zeros((L, n))
    lib().kso_continuum(
        C.c_int64(L), _p(_d(grid), P_D), C.c_int64(n), _p(wledge, P_D),
        _p(_d(atm["half_edge"]), P_D), _p(_d(atm["delta_edge"]), P_D), C.c_int64(wledge.size),
        _p(_d(atm["cont_abs_coeff"]), P_D), _p(_d(atm["cont_scat_coeff"]), P_D),
        C.c_int(int(bool(atm["cont_coeff_log10"]))), _p(ca, P_D), _p(cs, P_D))
    return ca, cs


def txnxn(atm: Dict[str, np.ndarray]) -> np.ndarray:
    L = atm["temperature"].size
    out = np.zeros(L)
    lib().kso_txnxn(C.c_int64(L), _p(_d(atm["temperature"]), P_D), _p(_d(atm["xnf_h"]), P_D),
                    _p(_d(atm["xnf_he1"]), P_D), _p(_d(atm["xnf_h2"]), P_D), _p(out, P_D))
    return out


def transp(cat, route, atm, center_idx, cont_kapmin, tb, cutoff=1e-3, microturb=0.0):
    nl = cat["wavelength"].size
    L = atm["temperature"].size
    pop = _d(atm["population_per_ion"]); dop = _d(atm["doppler_per_ion"])
    nion, nelem = pop.shape[1], pop.shape[2]
    tr = np.zeros((nl, L)); valid = np.zeros((nl, L), dtype=np.uint8)
    txn = txnxn(atm)
    lib().kso_transp(
        C.c_int64(nl), C.c_int64(L), _p(route["process_mask"], P_U8),
        _p(np.ascontiguousarray(route["element_idx"], np.int32), P_I32),
        _p(np.ascontiguousarray(cat["ion_stage"], np.int32), P_I32),
        _p(np.ascontiguousarray(cat["line_type"], np.int32), P_I32),
        _p(_d(cat["wavelength"]), P_D), _p(_d(route["gf"]), P_D), _p(_d(route["cgf"]), P_D),
        _p(_d(cat["gamma_rad"]), P_D), _p(_d(cat["gamma_stark"]), P_D), _p(_d(cat["gamma_vdw"]), P_D),
        _p(_d(cat["excitation_energy"]), P_D), _p(np.ascontiguousarray(center_idx, np.int64), P_I64),
        _p(_d(atm["hckt"]), P_D), _p(pop, P_D), _p(dop, P_D), C.c_int64(nion), C.c_int64(nelem),
        _p(_d(atm["mass_density"]), P_D), _p(_d(atm["electron_density"]), P_D), _p(txn, P_D),
        _p(_d(cont_kapmin), P_D), C.c_int64(cont_kapmin.shape[1]), C.c_double(cutoff),
        C.c_double(microturb), _p(tb["h0tab"], P_D), _p(tb["h1tab"], P_D), _p(tb["h2tab"], P_D),
        _p(tb["extab"], P_D), _p(tb["extabf"], P_D), _p(tr, P_D), _p(valid, P_U8))
    return tr, valid.astype(bool)


def asynth(cat, route, atm, grid, tr, valid, center_idx, wing_idx, cont_kapmin, tb, cutoff=1e-3):
    nl = cat["wavelength"].size
    L = atm["temperature"].size
    n = grid.size
    dop = _d(atm["doppler_per_ion"])
    nion, nelem = dop.shape[1], dop.shape[2]
    out = np.zeros((L, n))
    evals = np.zeros(L, dtype=np.int64)
    reach = np.zeros((nl, L), dtype=np.int32)
    lib().kso_asynth(
        C.c_int64(nl), C.c_int64(L), _p(np.ascontiguousarray(valid, np.uint8), P_U8), _p(_d(tr), P_D),
        _p(np.ascontiguousarray(cat["line_type"], np.int32), P_I32), _p(route["asynth_mask"], P_U8),
        _p(np.ascontiguousarray(cat["ion_stage"], np.int32), P_I32),
        _p(np.ascontiguousarray(route["element_idx"], np.int32), P_I32),
        _p(_d(cat["wavelength"]), P_D), _p(np.ascontiguousarray(center_idx, np.int64), P_I64),
        _p(np.ascontiguousarray(wing_idx, np.int64), P_I64),
        _p(_d(cat["gamma_rad"]), P_D), _p(_d(cat["gamma_stark"]), P_D), _p(_d(cat["gamma_vdw"]), P_D),
        _p(dop, P_D), C.c_int64(nion), C.c_int64(nelem), _p(_d(atm["electron_density"]), P_D),
        _p(txnxn(atm), P_D), _p(_d(atm["temperature"]), P_D), _p(_d(cont_kapmin), P_D),
        _p(_d(grid), P_D), C.c_int64(n), C.c_double(cutoff),
        _p(tb["h0tab"], P_D), _p(tb["h1tab"], P_D), _p(tb["h2tab"], P_D), _p(out, P_D), _p(evals, P_I64),
        _p(reach, P_I32))
    return out, evals, reach


def line_source(atm, grid):
    L = atm["temperature"].size
    out = np.zeros((L, grid.size))
    lib().kso_line_source(C.c_int64(L), C.c_int64(grid.size), _p(_d(grid), P_D),
                          _p(_d(atm["temperature"]), P_D), _p(out, P_D))
    return out


def transfer(atm, grid, cont_abs, cont_scat, line_opacity, line_scattering, line_src, tb):
    L = atm["temperature"].size
    n = grid.size
    ft = np.zeros(n); fc = np.zeros(n)
    iters = np.zeros((n, 2), dtype=np.int32)
    lib().kso_transfer(
        C.c_int64(L), C.c_int64(n), _p(_d(grid), P_D), _p(_d(atm["temperature"]), P_D),
        _p(_d(atm["depth"]), P_D), _p(_d(cont_abs), P_D), _p(_d(cont_scat), P_D),
        _p(_d(line_opacity), P_D), _p(_d(line_scattering), P_D),
        _p(_d(line_src), P_D) if line_src is not None else None,
        _p(_d(tb["xtau"]), P_D), _p(_d(tb["ch"]), P_D), _p(_d(tb["coefj"]), P_D),
        _p(ft, P_D), _p(fc, P_D), _p(iters, P_I32))
    return ft, fc, iters


def synthesize(atm: Dict[str, np.ndarray], cat: Dict[str, np.ndarray], wl_start: float,
               wl_end: float, resolution: float = 300000.0, cutoff: float = 1e-3,
               microturb: float = 0.0, rhoxj: float = 0.0, tb=None,
               timings: Optional[Dict[str, float]] = None) -> Dict[str, np.ndarray]:
    """Whole LTE synthesis on the CPU: plain lines, and the hydrogen lines'
    HPROF4 profiles when the catalog holds any.  ``cat`` must already be
    window-filtered (``gfall.filter_window``)."""
    from . import gfall

    tb = tb or tables()
    t0 = time.perf_counter()
    grid = wavelength_grid(wl_start, wl_end, resolution)
    route = gfall.routing(cat)
    cidx = center_indices(grid, cat["wavelength"])
    widx = wing_indices(grid, cat["wavelength"], float(grid[0]))
    ca, cs = continuum(atm, grid)
    kapmin = ca + cs
    t1 = time.perf_counter()
    tr, valid = transp(cat, route, atm, cidx, kapmin, tb, cutoff, microturb)
    t2 = time.perf_counter()
    asy, evals, reach = asynth(cat, route, atm, grid, tr, valid, cidx, widx, kapmin, tb, cutoff)
    from . import fort19
    if fort19.normal_rows(cat).size or fort19.aut_rows(cat).size or fort19.cont_rows(cat).size:
        # fort.19 NORMAL and autoionizing lines: their profiles added to ASYNTH
        # (synthe_py/engine/opacity.py:2366-2390)
        asy = asy + fort19.asynth_term(dict(cat, center=cidx), atm, grid, kapmin, cutoff=cutoff,
                                       microturb_kms=microturb)
    t3 = time.perf_counter()
    rhox = np.asarray(atm["depth"], dtype=np.float64)
    fscat = np.exp(-rhox / rhoxj) if rhoxj > 0.0 else np.zeros_like(rhox)
    line_op = asy * (1.0 - fscat[:, None])
    line_sc = asy * fscat[:, None]
    extra = {}
    lt = np.asarray(cat["line_type"])
    if np.any(((lt == -1) | (lt == -2)) & (np.asarray(cat["ion_stage"]) == 1)):
        # hydrogen lines: AHLINE added to the line opacity
        # (synthe_py/engine/opacity.py:2465-2503)
        from . import hydrogen
        hc = dict(wavelength=cat["wavelength"], gf=10.0 ** cat["log_gf"], elo=cat["excitation_energy"],
                  n_lower=cat["n_lower"], n_upper=cat["n_upper"], line_type=lt,
                  ion_stage=cat["ion_stage"], center=cidx)
        ah = hydrogen.line_opacity(hc, atm, grid, kapmin, cutoff=cutoff, microturb_kms=microturb)
        line_op = line_op + ah * (1.0 - fscat[:, None])
        line_sc = (asy + ah) * fscat[:, None]
        extra = dict(ahline=ah, line_opacity=line_op)
    if np.any(np.isin(lt, (-3, -4, -6))):
        # helium lines: AHE x STIM added to the line opacity
        # (synthe_py/engine/opacity.py:3650-3660)
        from . import helium
        ec = dict(wavelength=cat["wavelength"], gf=10.0 ** cat["log_gf"], elo=cat["excitation_energy"],
                  gamma_rad=cat["gamma_rad"], gamma_stark=cat["gamma_stark"], gamma_vdw=cat["gamma_vdw"],
                  ion_stage=cat["ion_stage"], line_type=lt, center=cidx, code=cat["code"],
                  n_lower=cat["n_lower"], n_upper=cat["n_upper"])
        for k in ("iso1", "iso2"):
            if k in cat:
                ec[k] = cat[k]
        he = helium.line_opacity(ec, atm, grid, kapmin, cutoff=cutoff)
        line_op = line_op + he * (1.0 - fscat[:, None])
        line_sc = line_sc + he * fscat[:, None]
        extra = dict(extra, ahe_stim=he, line_opacity=line_op)
    src = line_source(atm, grid)
    ft, fc, iters = transfer(atm, grid, ca, cs, line_op, line_sc, src, tb)
    t4 = time.perf_counter()
    conv = 2.99792458e17 / np.maximum(grid ** 2, 1e-40)
    if timings is not None:
        timings.update(setup=t1 - t0, transp=t2 - t1, asynth=t3 - t2, transfer=t4 - t3)
    return dict(
        wavelength=grid, center_indices=cidx, wing_indices=widx, cont_abs=ca, cont_scat=cs,
        transp=tr, valid_mask=valid, asynth=asy, evals_per_depth=evals, reach=reach,
        flux_total_hz=ft, flux_cont_hz=fc, flux_total=ft * conv, flux_cont=fc * conv,
        iterations=iters, **extra,
    )


def load_atmosphere(path: Path) -> Dict[str, np.ndarray]:
    with np.load(path) as d:
        return {k: np.asarray(d[k]) for k in d}
