"""Many syntheses as one batch: the batched form.

Each job is one atmosphere (its own layer count) and one wavelength window
(its own grid); all jobs share one line list resident in HBM.  The list is
sorted by wavelength, so the lines inside a job's DELLIM window
(synthe_py/io/lines/atomic.py:762-816, one margin for every non-hydrogen
line) are a contiguous slice of it, handed to the library as a row range
(no copy).  :class:`BatchSynthesizer` makes one batch plan
(``ks_batch_create``): every stage of the synthesis -- bins, per-depth
state, continuum, TRANSP and wing setup, reach-class partition, accumulation,
transfer -- runs as one persistent launch over all jobs (15 launches per
batch, whatever the number of jobs), the blocks walking a device table of
(job, block) work items.  :meth:`BatchSynthesizer.capture` records the batch
as a CUDA graph and :meth:`BatchSynthesizer.replay` launches it.  The tile
width, warps per tile and the pairs dealt to a warp at once come from
:mod:`kurucz_py_joss_submission_gb300.autotune`.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import _native
from .device import DeviceAtmosphere, DeviceCatalog, DeviceGrid, _ptr, check_flags, make_options, stream_handle
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


class BatchSynthesizer:
    """Fused syntheses of ``jobs`` over the shared lines of ``catalog``, as
    batch plans.  ``options`` (keywords of :func:`device.make_options`, e.g.
    from :func:`autotune.tune`) apply to every job.  With ``groups`` > 1 the
    jobs are dealt (largest first) to that many plans, each run on a stream of
    its own, so that one group's compute-bound transfer overlaps another's
    latency-bound pair setup; every group is still one persistent launch per
    stage."""

    def __init__(self, catalog: DeviceCatalog, atmospheres: Sequence[AtmosphereModel], jobs: Sequence[Job],
                 precision: str = "mixed", resolution: float = 300000.0, options: Optional[dict] = None,
                 workspace: Optional[torch.Tensor] = None, groups: int = 1, device="cuda"):
        host = catalog.host
        if np.any((np.abs(host.code - 1.0) < 1e-6) | np.isin(host.line_types, [-1, -2]) |
                  (host.element_idx == 0)):
            raise ValueError("BatchSynthesizer: line lists with hydrogen lines need per-job catalogs")
        if catalog.order is not None:
            raise ValueError("BatchSynthesizer: the shared catalog must be sorted by wavelength")
        self.lib = _native.load()
        self.catalog = catalog
        self.jobs = list(jobs)
        self.precision = precision
        self.option_keys = dict(options or {})
        self.options = make_options(precision=precision, **self.option_keys)
        self.atm = [DeviceAtmosphere(a, device=device) for a in atmospheres]
        self.grids: List[DeviceGrid] = []
        self.rows: List[slice] = []
        self.flux_total: List[torch.Tensor] = []
        self.flux_cont: List[torch.Tensor] = []
        wl_sorted = np.asarray(host.wavelength)
        for j in self.jobs:
            g = DeviceGrid(wavelength_grid(j.wl_start, j.wl_end, resolution), device=device)
            self.grids.append(g)
            self.rows.append(window_slice(wl_sorted, j.wl_start, j.wl_end))
            self.flux_total.append(torch.empty(g.n, dtype=torch.float64, device=g.wavelength.device))
            self.flux_cont.append(torch.empty(g.n, dtype=torch.float64, device=g.wavelength.device))
        n = len(self.jobs)
        self.job_recs = (_native.KsJob * n)()
        for i, j in enumerate(self.jobs):
            r = self.job_recs[i]
            r.atm = C.pointer(self.atm[j.atmosphere].rec)
            r.grid = C.pointer(self.grids[i].rec)
            r.line_first = self.rows[i].start
            r.line_count = self.rows[i].stop - self.rows[i].start
            r.flux_total = self.flux_total[i].data_ptr()
            r.flux_cont = self.flux_cont[i].data_ptr()
        # groups: jobs dealt round-robin in order of their work (lines x points)
        self.n_groups = max(1, min(int(groups), n))
        cost = [(self.rows[i].stop - self.rows[i].start) * self.grids[i].n for i in range(n)]
        order = sorted(range(n), key=lambda i: -cost[i])
        self.group_jobs = [sorted(order[g::self.n_groups]) for g in range(self.n_groups)]
        self.group_recs, sizes = [], []
        for members in self.group_jobs:
            recs = (_native.KsJob * len(members))(*[self.job_recs[i] for i in members])
            ws = C.c_size_t()
            _native.check(self.lib.ks_batch_workspace_size(C.byref(catalog.rec), recs, len(members),
                                                           C.byref(self.options), C.byref(ws)))
            self.group_recs.append(recs)
            sizes.append((int(ws.value) + 511) // 512 * 512)
        dev = self.grids[0].wavelength.device if self.grids else torch.device(device)
        self.workspace_bytes = sum(sizes)
        if workspace is not None and workspace.numel() >= self.workspace_bytes:
            self.workspace = workspace  # the caller's (e.g. shared by the autotuner's candidates)
        else:
            self.workspace = torch.empty(self.workspace_bytes, dtype=torch.uint8, device=dev)
        self.plans: List[C.c_void_p] = []
        off = 0
        for recs, size in zip(self.group_recs, sizes):
            plan = C.c_void_p()
            _native.check(self.lib.ks_batch_create(C.byref(catalog.rec), recs, len(recs), C.byref(self.options),
                                                   C.c_void_p(self.workspace.data_ptr() + off), size,
                                                   C.byref(plan)))
            self.plans.append(plan)
            off += size
        self.streams = [torch.cuda.Stream(device=dev) for _ in range(self.n_groups)] if self.n_groups > 1 else []
        self.graph: Optional[torch.cuda.CUDAGraph] = None

    def __del__(self):
        for plan in getattr(self, "plans", []):
            if plan is not None and plan.value:
                self.lib.ks_batch_free(plan)
        self.plans = []

    def run(self, stats: bool = False, stream: Optional[torch.cuda.Stream] = None):
        """Enqueue the batch on the current stream (groups fork to their own
        streams and join back); with ``stats`` synchronise and return the
        counters summed over the jobs."""
        if stats:
            tot = None
            for plan in self.plans:
                st = _native.KsStats()
                _native.check(self.lib.ks_batch_run(plan, C.byref(st), stream_handle(stream)))
                d = st.as_dict()
                if tot is None:
                    tot = d
                else:
                    for k in ("valid_pairs", "evaluations", "maxj_wavelengths", "iterations", "kernel_launches"):
                        tot[k] += d[k]
                    tot["device_flags"] |= d["device_flags"]
                    tot["stage_ms"] = {k: tot["stage_ms"][k] + d["stage_ms"][k] for k in tot["stage_ms"]}
            return tot
        if self.n_groups == 1:
            _native.check(self.lib.ks_batch_run(self.plans[0], None, stream_handle(stream)))
            return None
        cur = stream if stream is not None else torch.cuda.current_stream()
        for plan, s in zip(self.plans, self.streams):
            s.wait_stream(cur)
            _native.check(self.lib.ks_batch_run(plan, None, C.c_void_p(s.cuda_stream)))
        for s in self.streams:
            cur.wait_stream(s)
        return None

    def capture(self):
        """Record the batch as one CUDA graph (after one eager run, which
        also uploads the library's tables to this device)."""
        self.run()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, capture_error_mode="thread_local"):
            self.run()
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
        """Total line.depth.lambda evaluations of the batch (one synchronous run)."""
        return int(self.run(stats=True)["evaluations"])


def bucket(n: int) -> int:
    """Size class of a grid (powers of 4 points)."""
    b = 0
    while n > 1024 and b < 8:
        n //= 4
        b += 1
    return b
