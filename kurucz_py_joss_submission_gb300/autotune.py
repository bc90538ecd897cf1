"""Autotuner of the accumulation's launch shape.

The accumulation kernel's tile width (bins per CTA) and warps per tile trade
per-CTA fixed costs (staging the Voigt table, class ranges, the epilogue)
against occupancy and the number of tiles a long wing is read by; the best
choice depends on the grid size and the line density.  ``tune`` times each
candidate on a representative job with the library's own stage timers
(CUDA events on the launching stream) and keeps the fastest; results are
cached per (device name, precision, size class) in a JSON file next to the
built library.
"""

from __future__ import annotations

import ctypes as C
import json
import os
from pathlib import Path
from typing import Dict, Optional

import torch

from . import _build, _native
from .device import _ptr, make_options

CANDIDATES = [dict(tile_bins=t, warps_per_tile=w) for t in (256, 512, 1024) for w in (4, 8)]
CACHE = Path(os.environ.get("KS_AUTOTUNE_CACHE", str(_build.OUT_DIR / "autotune.json")))


def _time_total(lib, view, atm_rec, grid_rec, opt, ws: torch.Tensor, ft, fc, reps: int) -> float:
    best = float("inf")
    for _ in range(reps):
        st = _native.KsStats()
        _native.check(lib.ks_synthesize(C.byref(view), C.byref(atm_rec), C.byref(grid_rec), C.byref(opt),
                                        _ptr(ws), ws.numel(), _ptr(ft), _ptr(fc), None, C.byref(st), None))
        best = min(best, float(st.stage_ms[7]))
    return best


def _load_cache() -> dict:
    try:
        return json.loads(CACHE.read_text())
    except (OSError, ValueError):
        return {}


def tune(batch, reps: int = 3, use_cache: bool = True) -> Dict[int, dict]:
    """Best candidate per size class of ``batch`` (a BatchSynthesizer built
    without tuned options); returns {size class: options}."""
    from .batch import bucket

    lib = _native.load()
    dev = torch.cuda.get_device_name()
    cache = _load_cache() if use_cache else {}
    reps_job: Dict[int, int] = {}
    for i, g in enumerate(batch.grids):
        b = bucket(g.n)
        if b not in reps_job or batch.views[i].n_lines > batch.views[reps_job[b]].n_lines:
            reps_job[b] = i
    out: Dict[int, dict] = {}
    for b, i in sorted(reps_job.items()):
        key = f"{dev}|{batch.precision}|{b}"
        if key in cache:
            out[b] = cache[key]
            continue
        j = batch.jobs[i]
        best, best_t = None, float("inf")
        for cand in CANDIDATES:
            opt = make_options(precision=batch.precision, profile=True, **cand)
            ws_n = C.c_size_t()
            _native.check(lib.ks_workspace_size(batch.views[i].n_lines, batch.atm[j.atmosphere].n_layers,
                                                batch.grids[i].n, C.byref(opt), C.byref(ws_n)))
            ws = torch.empty(int(ws_n.value), dtype=torch.uint8, device=batch.grids[i].wavelength.device)
            t = _time_total(lib, batch.views[i], batch.atm[j.atmosphere].rec, batch.grids[i].rec, opt, ws,
                            batch.flux_total[i], batch.flux_cont[i], reps)
            if t < best_t:
                best, best_t = cand, t
            del ws
        out[b] = dict(best)
        cache[key] = dict(best)
    if use_cache:
        try:
            CACHE.parent.mkdir(parents=True, exist_ok=True)
            CACHE.write_text(json.dumps(cache, indent=1))
        except OSError:
            pass
    return out
