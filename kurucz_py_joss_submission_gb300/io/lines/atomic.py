"""gfall line catalogs through the native reader.

``load_catalog`` mirrors synthe_py/io/lines/atomic.py:299 (fixed-width and
whitespace records, damping defaults, 4*pi*nu normalisation, line types) and
``filter_by_range`` its :762 DELLIM window.  The catalog is a struct of
arrays; ``process_mask``/``asynth_mask`` carry the TRANSP routing of
synthe_py/physics/line_opacity.py:740-765 and the ASYNTH centre classes of
:1094.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, fields
from pathlib import Path
from typing import Optional

import numpy as np

from ... import _native

DELLIM = np.array([100.0, 30.0, 10.0, 3.0, 1.0, 0.3, 0.1])


@dataclass
class LineCatalog:
    wavelength: np.ndarray
    log_gf: np.ndarray
    gf: np.ndarray
    cgf: np.ndarray
    excitation_energy: np.ndarray
    gamma_rad: np.ndarray
    gamma_stark: np.ndarray
    gamma_vdw: np.ndarray
    element_idx: np.ndarray
    ion_stages: np.ndarray
    line_types: np.ndarray
    process_mask: np.ndarray
    asynth_mask: np.ndarray
    code: np.ndarray
    catalog_index: np.ndarray
    n_lower: np.ndarray   # NBLO: lower principal quantum number (hydrogen lines), 0 if blank
    n_upper: np.ndarray   # NBUP
    iso1: np.ndarray      # ISO1 / ISO2 (isotope numbers; ISO2 doubles as fort.19's continuum index)
    iso2: np.ndarray
    gamma_rad_log: np.ndarray    # GR / GS / GW as read (log10, 0 when blank)
    gamma_stark_log: np.ndarray
    gamma_vdw_log: np.ndarray
    xj: np.ndarray               # J of the lower / upper level
    xjp: np.ndarray
    continuum_label: np.ndarray  # 1 where LABELP begins with CONTINUU (merged-continuum record)

    def __len__(self) -> int:
        return int(self.wavelength.size)

    @property
    def index_wavelength(self) -> np.ndarray:
        return self.wavelength

    def take(self, idx: np.ndarray) -> "LineCatalog":
        return LineCatalog(**{f.name: getattr(self, f.name)[idx] for f in fields(self)})

    def is_sorted(self) -> bool:
        w = self.wavelength
        return bool(w.size < 2 or np.all(w[1:] >= w[:-1]))


_POTION: Optional[np.ndarray] = None


def _potion() -> np.ndarray:
    global _POTION
    if _POTION is None:
        with np.load(_native.TABLES_NPZ) as t:
            _POTION = np.ascontiguousarray(t["potion"], dtype=np.float64)
    return _POTION


def _read(path: Path, wl_min: float, wl_max: float, sort: bool) -> LineCatalog:
    L = _native.load()
    pot = _potion()
    h = C.c_void_p()
    st = L.ks_gfall_read(str(path).encode(), float(wl_min), float(wl_max),
                         pot.ctypes.data_as(_native.PD), pot.size, C.byref(h))
    if st != 0:
        if st == 5:
            raise FileNotFoundError(str(path))
        _native.check(st)
    try:
        if sort:
            _native.check(L.ks_gfall_sort(h))
        n = int(L.ks_gfall_count(h))
        cols = dict(
            wavelength=np.zeros(n), log_gf=np.zeros(n), gf=np.zeros(n), cgf=np.zeros(n),
            excitation_energy=np.zeros(n), gamma_rad=np.zeros(n), gamma_stark=np.zeros(n),
            gamma_vdw=np.zeros(n), element_idx=np.zeros(n, np.int32), ion_stages=np.zeros(n, np.int32),
            line_types=np.zeros(n, np.int32), process_mask=np.zeros(n, np.uint8),
            asynth_mask=np.zeros(n, np.uint8), code=np.zeros(n), catalog_index=np.zeros(n, np.int64),
            n_lower=np.zeros(n, np.int32), n_upper=np.zeros(n, np.int32),
            iso1=np.zeros(n, np.int32), iso2=np.zeros(n, np.int32),
            gamma_rad_log=np.zeros(n), gamma_stark_log=np.zeros(n), gamma_vdw_log=np.zeros(n),
            xj=np.zeros(n), xjp=np.zeros(n), continuum_label=np.zeros(n, np.uint8),
        )
        order = ["wavelength", "log_gf", "gf", "cgf", "excitation_energy", "gamma_rad", "gamma_stark",
                 "gamma_vdw", "element_idx", "ion_stages", "line_types", "process_mask",
                 "asynth_mask", "code", "catalog_index"]
        _native.check(L.ks_gfall_fetch(h, *[cols[k].ctypes.data_as(C.c_void_p) for k in order]))
        _native.check(L.ks_gfall_fetch_levels(h, cols["n_lower"].ctypes.data_as(C.c_void_p),
                                              cols["n_upper"].ctypes.data_as(C.c_void_p)))
        _native.check(L.ks_gfall_fetch_iso(h, cols["iso1"].ctypes.data_as(C.c_void_p),
                                           cols["iso2"].ctypes.data_as(C.c_void_p)))
        _native.check(L.ks_gfall_fetch_gamma_logs(h, *[cols[k].ctypes.data_as(C.c_void_p) for k in
                                                       ("gamma_rad_log", "gamma_stark_log", "gamma_vdw_log")]))
        _native.check(L.ks_gfall_fetch_j(h, *[cols[k].ctypes.data_as(C.c_void_p) for k in
                                              ("xj", "xjp", "continuum_label")]))
    finally:
        L.ks_gfall_free(h)
    return LineCatalog(**cols)


def load_catalog(path: Path) -> LineCatalog:
    """Every record of a gfall file, in file order."""
    return _read(Path(path), 0.0, 0.0, sort=False)


def load_catalog_window(path: Path, wl_min: float, wl_max: float, sort: bool = False) -> LineCatalog:
    """Records inside the DELLIM window of [wl_min, wl_max], read natively."""
    return _read(Path(path), wl_min, wl_max, sort=sort)


def filter_by_range(catalog: LineCatalog, wl_min: float, wl_max: float) -> LineCatalog:
    """atomic.py:762-816: keep lines within DELLIM(LIM)*DELFACTOR of the window."""
    delfactor = 1.0 if wl_min <= 500.0 else wl_min / 500.0
    lim = np.full(len(catalog), 7)
    hmask = (np.abs(catalog.code - 1.0) < 1e-6) | np.isin(catalog.line_types, [-1, -2]) | (
        catalog.element_idx == 0)
    lim = np.where(hmask, 1, lim)
    margin = DELLIM[lim - 1] * delfactor
    w = catalog.wavelength
    keep = np.nonzero((w >= wl_min - margin) & (w <= wl_max + margin))[0]
    return catalog.take(keep)
