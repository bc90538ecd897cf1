"""Many syntheses in one captured CUDA graph: the batched form.

Each job is one atmosphere (its own layer count) and one wavelength window
(its own grid); all jobs share one line list resident in HBM.  The list is
sorted by wavelength, so the lines inside a job's DELLIM window
(synthe_py/io/lines/atomic.py:762-816, one margin for every non-hydrogen
line) are a contiguous slice of it, handed to the library as a pointer view
(no copy).  Jobs are spread over several CUDA streams, each stream with one
workspace sized for its largest job; :meth:`BatchSynthesizer.capture`
records the whole batch -- every job's continuum, TRANSP, ASYNTH and
transfer launches on every stream -- as one CUDA graph, and
:meth:`BatchSynthesizer.replay` launches it.  Per-job tile options come from
:mod:`kurucz_py_joss_submission_gb300.autotune`.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import _native
from .device import DeviceAtmosphere, DeviceCatalog, DeviceGrid, _ptr, check_flags, make_options
from .io.atmosphere import AtmosphereModel
from .io.lines.atomic import DELLIM


@dataclass(frozen=True)
class Job:
    atmosphere: int      # index into the batch's atmospheres
    wl_start: float      # nm
    wl_end: float        # nm


def wavelength_grid(wl_start: float, wl_end: float, resolution: float = 300000.0) -> np.ndarray:
    """The reference's log-lambda grid (engine/opacity.py:526), from the library."""
    lib = _native.load()
    n = lib.ks_wavelength_grid(wl_start, wl_end, resolution, None, 0)
    g = np.zeros(n)
    lib.ks_wavelength_grid(wl_start, wl_end, resolution, g.ctypes.data_as(_native.PD), n)
    return g


def window_slice(wavelength_sorted: np.ndarray, wl_min: float, wl_max: float) -> slice:
    """Rows of a wavelength-sorted list without hydrogen lines inside the
    DELLIM window of [wl_min, wl_max] (LIM 7 margin, scaled by wl_min/500
    above 500 nm, as filter_by_range)."""
    delfactor = 1.0 if wl_min <= 500.0 else wl_min / 500.0
    margin = DELLIM[6] * delfactor
    i0 = int(np.searchsorted(wavelength_sorted, wl_min - margin, side="left"))
    i1 = int(np.searchsorted(wavelength_sorted, wl_max + margin, side="right"))
    return slice(i0, i1)


def lines_view(cat: DeviceCatalog, rows: slice) -> _native.KsLines:
    """A ks_lines record for rows [start, stop) of a device catalog."""
    i0, n = rows.start, rows.stop - rows.start
    rec = _native.KsLines()
    rec.n_lines = n

    def at(name, size):
        return cat.t[name].data_ptr() + i0 * size

    rec.wavelength = at("wavelength", 8)
    rec.gf = at("gf", 8)
    rec.cgf = at("cgf", 8)
    rec.gamma_rad = at("gamma_rad", 8)
    rec.gamma_stark = at("gamma_stark", 8)
    rec.gamma_vdw = at("gamma_vdw", 8)
    rec.elo_cm = at("excitation_energy", 8)
    rec.element_idx = at("element_idx", 4)
    rec.ion_stage = at("ion_stages", 4)
    rec.line_type = at("line_types", 4)
    rec.process_mask = at("process_mask", 1)
    rec.asynth_mask = at("asynth_mask", 1)
    rec.sorted_by_wavelength = 1
    return rec


class BatchSynthesizer:
    """Fused syntheses of ``jobs`` over shared lines, on ``n_streams`` streams."""

    def __init__(self, catalog: DeviceCatalog, atmospheres: Sequence[AtmosphereModel], jobs: Sequence[Job],
                 precision: str = "mixed", resolution: float = 300000.0, n_streams: int = 32,
                 tuned: Optional[Dict[int, dict]] = None, device="cuda"):
        host = catalog.host
        if np.any((np.abs(host.code - 1.0) < 1e-6) | np.isin(host.line_types, [-1, -2]) |
                  (host.element_idx == 0)):
            raise ValueError("BatchSynthesizer: line lists with hydrogen lines need per-job catalogs")
        self.lib = _native.load()
        self.catalog = catalog
        self.jobs = list(jobs)
        self.precision = precision
        self.atm = [DeviceAtmosphere(a, device=device) for a in atmospheres]
        self.grids: List[DeviceGrid] = []
        self.views: List[_native.KsLines] = []
        self.options: List[_native.KsOptions] = []
        self.flux_total: List[torch.Tensor] = []
        self.flux_cont: List[torch.Tensor] = []
        self.ws_bytes: List[int] = []
        wl_sorted = np.asarray(host.wavelength)
        tuned = tuned or {}
        for j in self.jobs:
            g = wavelength_grid(j.wl_start, j.wl_end, resolution)
            dg = DeviceGrid(g, device=device)
            rows = window_slice(wl_sorted, j.wl_start, j.wl_end)
            view = lines_view(catalog, rows)
            t = tuned.get(bucket(dg.n), {})
            opt = make_options(precision=precision, **t)
            ws = C.c_size_t()
            _native.check(self.lib.ks_workspace_size(view.n_lines, self.atm[j.atmosphere].n_layers, dg.n,
                                                     C.byref(opt), C.byref(ws)))
            self.grids.append(dg)
            self.views.append(view)
            self.options.append(opt)
            self.ws_bytes.append(int(ws.value))
            self.flux_total.append(torch.empty(dg.n, dtype=torch.float64, device=dg.wavelength.device))
            self.flux_cont.append(torch.empty(dg.n, dtype=torch.float64, device=dg.wavelength.device))
        # largest jobs first, dealt round-robin to the streams
        order = sorted(range(len(self.jobs)), key=lambda i: -self.ws_bytes[i])
        self.n_streams = max(1, min(n_streams, len(self.jobs)))
        self.assign: List[List[int]] = [order[s::self.n_streams] for s in range(self.n_streams)]
        dev = self.grids[0].wavelength.device if self.grids else torch.device(device)
        self.streams = [torch.cuda.Stream(device=dev) for _ in range(self.n_streams)]
        self.workspaces = [torch.empty(max([self.ws_bytes[i] for i in a] or [1]), dtype=torch.uint8, device=dev)
                           for a in self.assign]
        self.graph: Optional[torch.cuda.CUDAGraph] = None

    def _enqueue(self):
        cur = torch.cuda.current_stream()
        for s, stream in enumerate(self.streams):
            stream.wait_stream(cur)
            ws = self.workspaces[s]
            for i in self.assign[s]:
                status = self.lib.ks_synthesize(
                    C.byref(self.views[i]), C.byref(self.atm[self.jobs[i].atmosphere].rec),
                    C.byref(self.grids[i].rec), C.byref(self.options[i]), _ptr(ws), ws.numel(),
                    _ptr(self.flux_total[i]), _ptr(self.flux_cont[i]), None, None,
                    C.c_void_p(stream.cuda_stream))
                _native.check(status)
        for stream in self.streams:
            cur.wait_stream(stream)

    def run(self):
        """Enqueue every job on the current stream's device (no graph)."""
        self._enqueue()

    def capture(self):
        """Record the batch as one CUDA graph (after one eager run, which
        also uploads the library's tables to this device)."""
        self.run()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, capture_error_mode="thread_local"):
            self._enqueue()
        self.graph = g
        return g

    def replay(self, check: bool = False):
        """Launch the captured batch; with ``check`` wait for it and raise if
        any job flagged an internal limit (the flags stay on the device
        otherwise, until :func:`device.check_flags`)."""
        if self.graph is None:
            raise RuntimeError("capture() first")
        self.graph.replay()
        if check:
            check_flags()

    def evaluations(self) -> int:
        """Total line.depth.lambda evaluations of the batch (one synchronous pass)."""
        tot = 0
        for i, j in enumerate(self.jobs):
            st = _native.KsStats()
            ws = self.workspaces[next(s for s, a in enumerate(self.assign) if i in a)]
            _native.check(self.lib.ks_synthesize(
                C.byref(self.views[i]), C.byref(self.atm[j.atmosphere].rec), C.byref(self.grids[i].rec),
                C.byref(self.options[i]), _ptr(ws), ws.numel(), _ptr(self.flux_total[i]),
                _ptr(self.flux_cont[i]), None, C.byref(st), None))
            tot += int(st.evaluations)
        return tot


def bucket(n: int) -> int:
    """Size class of a job's grid for the tuned options (powers of 4 points)."""
    b = 0
    while n > 1024 and b < 8:
        n //= 4
        b += 1
    return b
