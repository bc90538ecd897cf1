"""Autotuner of the batched form's launch shape.

The accumulation's tile width (bins per CTA), its warps per tile, the
number of long-reach pairs dealt to a warp at once (``long_class``: classes
from it go in batches of 8 pairs, the shorter ones in batches of 32) and the
number of job groups run side by side (``groups``) trade
per-CTA fixed costs (staging the Voigt table, class ranges, the epilogue)
against occupancy, load balance and the number of tiles a long wing is read
by; the best choice depends on the grid sizes and the line density of the
batch.  :func:`tune` builds the batch plan for each candidate (sharing one
workspace), times whole batch runs with CUDA events on the launching stream
and keeps the fastest; results are cached per (device name, precision,
batch signature) in a JSON file next to the built library.
"""

from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path
from typing import Callable, Optional

import torch

from . import _build

CANDIDATES = ([dict(tile_bins=t, warps_per_tile=w, long_class=lc) for t in (512, 1024) for w in (4, 8)
               for lc in (8, 10)] + [dict(tile_bins=2048, warps_per_tile=8, long_class=lc) for lc in (8, 10)])
# job groups: plans run side by side on streams of their own
GROUPS = (2, 4, 8)
CACHE = Path(os.environ.get("KS_AUTOTUNE_CACHE", str(_build.OUT_DIR / "autotune.json")))


def _load_cache() -> dict:
    try:
        return json.loads(CACHE.read_text())
    except (OSError, ValueError):
        return {}


def signature(jobs, n_lines: int, layers) -> str:
    """A key for a batch: its jobs' windows and atmospheres and the list size."""
    h = hashlib.sha256()
    h.update(repr((n_lines, [(j.atmosphere, round(j.wl_start, 6), round(j.wl_end, 6)) for j in jobs],
                   list(layers))).encode())
    return h.hexdigest()[:16]


def time_batch(bs, reps: int = 3) -> float:
    """Best of ``reps`` runs of a batch plan, ms (CUDA events on the current stream)."""
    bs.run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = float("inf")
    for _ in range(reps):
        e0.record()
        bs.run()
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def tune(make_batch: Callable[..., object], key: str, precision: str, reps: int = 3,
         use_cache: bool = True, log: Optional[Callable[[str], None]] = None) -> dict:
    """The fastest candidate for a batch.  ``make_batch(options, workspace)``
    builds the BatchSynthesizer with the given options (a dict of
    make_options keywords) over the given workspace (None: allocate); ``key``
    identifies the batch (see :func:`signature`)."""
    dev = torch.cuda.get_device_name()
    cache = _load_cache() if use_cache else {}
    ck = f"{dev}|{precision}|{key}"
    if ck in cache:
        return dict(cache[ck])
    ws = None
    best, best_t = None, float("inf")
    for cand in CANDIDATES:
        bs = make_batch(cand, ws)
        if ws is None or bs.workspace.numel() > ws.numel():
            ws = bs.workspace
        t = time_batch(bs, reps)
        if log:
            log(f"autotune {cand}: {t:.3f} ms")
        if t < best_t:
            best, best_t = dict(cand), t
        del bs
    # then the number of job groups (plans on streams of their own) for it
    best_g, best_gt = 1, best_t
    for groups in GROUPS:
        bs = make_batch(dict(best, groups=groups), ws)
        if bs.workspace.numel() > ws.numel():
            ws = bs.workspace
        t = time_batch(bs, reps)
        if log:
            log(f"autotune {best} x {groups} groups: {t:.3f} ms")
        if t < best_gt:
            best_g, best_gt = groups, t
        del bs
    best = dict(best, groups=best_g)
    if use_cache:
        cache[ck] = best
        try:
            CACHE.parent.mkdir(parents=True, exist_ok=True)
            CACHE.write_text(json.dumps(cache, indent=1))
        except OSError:
            pass
    return best
