"""Benchmark of the GB300 line-opacity + transfer path (one JSON line).

Workload (``--workload``, default ``full_300_1800``): one synthetic grey
atmosphere (Teff 5800 K, log g 4.44, 72 layers, converted by the reference's
own converter), the 300-1800 nm grid at R = 300000 (537,529 points) and 1.5M
seeded atomic lines (gfall format, log-uniform in wavelength).
``window_500_510`` is the 20,000-line 500-510 nm case (5,941 points) the
reference itself runs on a CPU; ``dense_10m`` the stress case: Teff 2500 K,
log g -1.0, 300-1800 nm, 1.5M atomic + 8.5M molecular-band-like lines.  A step is one full synthesis --
continuum, TRANSP, ASYNTH, line source, JOSH flux and continuum flux for
every grid point -- with inputs resident in HBM.  The metric is
line.depth.lambda evaluations per second (the exact count of opacity
contributions accumulated, as the reference's wing loops count them); the
line also carries spectra/s, ``e2e`` (same metric through the public API
from pinned host buffers, every step's copies inside the timed region; on
one GPU the next step's copies overlap the current synthesis), the live
roofline of the dominant kernel and the CPU baseline.

``--impl reference`` times the CPU restatement of the reference path
(``oracle/``, C + OpenMP on every host core) on a bounded sample of the
same workload; the reference itself is pure Python/Numba and cannot run on
the GPU host.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# Workloads: line draws from kurucz_py_joss_submission_gb300.workloads.WORKLOADS, plus the
# converted atmosphere and the CPU-baseline sample windows.
_SAMPLE_40NM = [(float(a), float(a) + 40.0) for a in np.exp(np.linspace(np.log(305.0), np.log(1750.0), 12))]
_SAMPLE_10NM = [(float(a), float(a) + 10.0) for a in np.exp(np.linspace(np.log(305.0), np.log(1780.0), 12))]
BENCH_WORKLOADS = {
    "full_300_1800": dict(atm="atm_t5800g444.npz", sample=_SAMPLE_40NM),
    "window_500_510": dict(atm="atm_t5800g444.npz", sample=[(500.0, 510.0)]),
    "dense_10m": dict(atm="atm_t2500gm10.npz", sample=_SAMPLE_10NM),
}
# Batched workload: 256 jobs (atmosphere, window) over the full_300_1800 line list
BATCH_JOBS, BATCH_SEED = 256, 304


def workload_spec(name: str) -> dict:
    from kurucz_py_joss_submission_gb300 import workloads

    spec = dict(workloads.WORKLOADS[name])
    spec.update(BENCH_WORKLOADS[name])
    spec["name"] = name
    spec.setdefault("resolution", 300000.0)
    return spec


WORKLOAD = workload_spec("full_300_1800")
METRIC = "line.depth.lambda evaluations/s (spectra/s alongside), <=1e-4 rel flux err vs FP64, 1xGB300"
# FP32 work per accumulated contribution: the far-wing value X/o^2 shared by
# the red and blue bin (1 mul + 1 fast divide = 2 flops per 2 contributions)
# plus the Kahan-compensated add (4 flops): 5 flops per contribution.
FLOPS_PER_EVAL = 5.0


def sample_text() -> str:
    w = WORKLOAD["sample"]
    return f"{len(w)} window(s) x {w[0][1] - w[0][0]:g} nm of the workload"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def workload_catalog_path() -> Path:
    from kurucz_py_joss_submission_gb300 import workloads

    tmp = Path(os.environ.get("TMPDIR", "/tmp"))
    p = tmp / f"kgb300_{WORKLOAD['name']}_{WORKLOAD['seed']}.gf"
    if not p.exists():
        t = time.time()
        d = workloads.random_atomic_lines(WORKLOAD["n_lines"], WORKLOAD["wl_start"], WORKLOAD["wl_end"],
                                          WORKLOAD["seed"], log_uniform=WORKLOAD["log_uniform"])
        if WORKLOAD.get("n_band_lines"):
            bands = workloads.random_band_lines(WORKLOAD["n_band_lines"], WORKLOAD["wl_start"],
                                                WORKLOAD["wl_end"], WORKLOAD["band_seed"])
            d = workloads.merge_lines(d, bands)
        tmpname = p.with_suffix(f".{os.getpid()}.tmp")
        workloads.write_gfall(tmpname, d)
        os.replace(tmpname, p)
        log(f"generated {p} in {time.time() - t:.1f}s")
    return p


def wavelength_grid(w0=None, w1=None):
    """The product's grid (ks_wavelength_grid); GPU arm only."""
    from kurucz_py_joss_submission_gb300 import _native

    w0 = WORKLOAD["wl_start"] if w0 is None else w0
    w1 = WORKLOAD["wl_end"] if w1 is None else w1
    L = _native.load()
    n = L.ks_wavelength_grid(w0, w1, WORKLOAD["resolution"], None, 0)
    g = np.zeros(n)
    L.ks_wavelength_grid(w0, w1, WORKLOAD["resolution"], g.ctypes.data_as(_native.PD), n)
    return g


def oracle_grid(w0=None, w1=None):
    """The oracle's restatement of the grid (opacity.py:526); CPU arm only."""
    from oracle import oracle

    w0 = WORKLOAD["wl_start"] if w0 is None else w0
    w1 = WORKLOAD["wl_end"] if w1 is None else w1
    return oracle.wavelength_grid(w0, w1, WORKLOAD["resolution"])


def _sha256(path: Path) -> str:
    import hashlib

    h = hashlib.sha256()
    with open(path, "rb") as f:
        for chunk in iter(lambda: f.read(1 << 24), b""):
            h.update(chunk)
    return h.hexdigest()


def oracle_sample_catalogs(cat_path: Path):
    """The sample windows of the workload read by the oracle's own gfall
    reader (``oracle/gfall.py``: parse, then the DELLIM window of each
    sample), in catalog order.  The restated reader takes about 12 s per 1.5M
    lines, so the windows are cached as one .npz in $TMPDIR keyed by the line
    file's sha256 and the sample; the cache is read before any timing."""
    from oracle import gfall

    windows = WORKLOAD["sample"]
    # the parser's field set is part of the key (a cache from an older reader lacks fields)
    tag = ("v3_" + _sha256(cat_path)[:20] + "_"
           + "_".join(f"{a:.3f}-{b:.3f}" for a, b in windows).replace(".", "p"))
    import hashlib

    cache = Path(os.environ.get("TMPDIR", "/tmp")) / f"kgb300_orcwin_{hashlib.sha256(tag.encode()).hexdigest()[:24]}.npz"
    if cache.exists():
        with np.load(cache) as z:
            cats = []
            for i in range(len(windows)):
                pre = f"w{i}__"
                cats.append({k[len(pre):]: np.asarray(z[k]) for k in z.files if k.startswith(pre)})
            return cats
    t = time.time()
    with np.load(ROOT / "kurucz_py_joss_submission_gb300" / "data" / "synthe_tables.npz") as d:
        potion = np.asarray(d["potion"])
    full = gfall.parse_gfall(cat_path, potion)
    cats = [gfall.filter_window(full, w0, w1) for w0, w1 in windows]
    tmp = cache.with_suffix(f".{os.getpid()}.tmp.npz")
    np.savez(tmp, **{f"w{i}__{k}": v for i, c in enumerate(cats) for k, v in c.items()})
    os.replace(tmp, cache)
    log(f"oracle reader: {full['wavelength'].size} lines parsed, {len(windows)} windows cached "
        f"in {time.time() - t:.1f}s")
    return cats


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        return False

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """DRAM bytes per launch of the accumulation kernel from the committed ncu summary."""
    p = ROOT / "profiles" / "accumulate_kernel_full_300_1800.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch_full_size"):
            try:
                return float(line.split("=")[1].split()[0])
            except (IndexError, ValueError):
                return None
    return None


def cpu_baseline(cat_path: Path, steps: int = 1):
    """The oracle (C restatement of the reference path, OpenMP) on the sample
    windows with every host thread: evals/s, plus the fluxes of the first
    pass (F_nu per window) for the GPU-vs-oracle accuracy block.  Touches only
    ``oracle/``: lines from the restated gfall reader, grid from the restated
    grid routine."""
    from oracle import oracle

    oracle.build()
    tb = oracle.tables()
    atm = oracle.load_atmosphere(ROOT / "tests" / "golden" / WORKLOAD["atm"])
    cats = oracle_sample_catalogs(cat_path)
    # every host core this process may run on (torchrun sets OMP_NUM_THREADS=1)
    oracle.set_threads(len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count())
    threads = oracle.num_threads()
    tot_t, tot_e, tot_pts = 0.0, 0, 0
    rep = 0
    fluxes = []
    # at least `steps` passes over the sample, and at least 10 s of CPU time
    while rep < steps or (tot_t < 10.0 and rep < 1000):
        rep += 1
        for (w0, w1), c in zip(WORKLOAD["sample"], cats):
            t = time.perf_counter()
            r = oracle.synthesize(atm, c, w0, w1, WORKLOAD["resolution"], tb=tb)
            tot_t += time.perf_counter() - t
            tot_e += int(r["evals_per_depth"].sum())
            tot_pts += r["wavelength"].size
            if rep == 1:
                fluxes.append((r["flux_total_hz"], r["flux_cont_hz"], int(r["evals_per_depth"].sum())))
    return dict(evals_per_s=tot_e / tot_t, seconds=tot_t, evals=tot_e, points=tot_pts,
                threads=threads, passes=rep, fluxes=fluxes)


# Normalised fluxes below this are saturated line cores (the MAXJ = 1 branch
# leaves F at zero to the reference's own precision, ~1e-18 of the
# continuum); their error is measured relative to this floor.
NORM_FLUX_FLOOR = 1e-3


def flux_errors(ft, fc, rt, rc) -> dict:
    """Errors of one spectrum (ft, fc) against a reference (rt, rc), in the
    metric's unit: the relative error of the normalised flux F/Fc (against
    max(F/Fc, NORM_FLUX_FLOOR)), and the relative error of the continuum flux."""
    n, nr = ft / fc, rt / rc
    d = n - nr
    rel = np.abs(d) / np.maximum(np.abs(nr), NORM_FLUX_FLOOR)
    i = int(np.argmax(rel))
    return {"norm_flux_max_rel": float(rel[i]), "norm_flux_rel_rms": float(np.sqrt(np.mean(rel * rel))),
            "norm_flux_at_max_rel": float(nr[i]), "norm_flux_min": float(np.min(nr)),
            "norm_flux_floor": NORM_FLUX_FLOOR, "points_below_floor": int(np.sum(np.abs(nr) < NORM_FLUX_FLOOR)),
            "norm_flux_max_abs": float(np.max(np.abs(d))), "norm_flux_rms": float(np.sqrt(np.mean(d * d))),
            "cont_flux_max_rel": float(np.max(np.abs(fc / rc - 1.0))), "points": int(n.size)}


def merge_errors(parts: list) -> dict:
    """Worst case (max) over several spectra, RMS pooled by points."""
    if not parts:
        return None
    out = {}
    pts = np.array([p["points"] for p in parts], dtype=np.float64)
    worst = max(parts, key=lambda p: p["norm_flux_max_rel"])
    for k in ("norm_flux_max_rel", "norm_flux_max_abs", "cont_flux_max_rel"):
        out[k] = max(p[k] for p in parts)
    for k in ("norm_flux_rel_rms", "norm_flux_rms"):
        out[k] = float(np.sqrt(np.sum(pts * np.array([p[k] ** 2 for p in parts])) / pts.sum()))
    out["norm_flux_at_max_rel"] = worst["norm_flux_at_max_rel"]
    out["norm_flux_min"] = min(p["norm_flux_min"] for p in parts)
    out["norm_flux_floor"] = NORM_FLUX_FLOOR
    out["points_below_floor"] = int(sum(p["points_below_floor"] for p in parts))
    out["points"] = int(pts.sum())
    return out


def accuracy_vs_port(cat_path: Path, datm, cpu: dict, dev) -> dict:
    """The GPU path (mixed and FP64) against the oracle on the CPU baseline's
    sample windows: the same lines (each window's DELLIM selection), grid and
    atmosphere, synthesised independently on both sides."""
    import torch

    from kurucz_py_joss_submission_gb300.device import DeviceCatalog, DeviceGrid, Synthesizer, make_options
    from kurucz_py_joss_submission_gb300.io.lines import atomic

    res = {"mixed": [], "fp64": []}
    evals_equal = True
    for (w0, w1), (oft, ofc, oev) in zip(WORKLOAD["sample"], cpu["fluxes"]):
        cat = atomic.load_catalog_window(cat_path, w0, w1, sort=True)
        grid = wavelength_grid(w0, w1)
        if grid.size != oft.size:
            raise RuntimeError(f"grid of [{w0}, {w1}] differs from the oracle's ({grid.size} vs {oft.size})")
        dcat, dgrid = DeviceCatalog(cat, dev), DeviceGrid(grid, device=dev)
        for prec in res:
            syn = Synthesizer(dcat, datm, dgrid, make_options(precision=prec), keep_asynth=False)
            st = syn.run(stats=True)
            if prec == "fp64":  # the FP64 gates are the reference's; FP32 ones may differ at the cutoff
                evals_equal &= int(st["evaluations"]) == oev
            res[prec].append(flux_errors(syn.flux_total.cpu().numpy(), syn.flux_cont.cpu().numpy(), oft, ofc))
            del syn
        del dcat, dgrid
    torch.cuda.synchronize()
    out = {k: merge_errors(v) for k, v in res.items()}
    out["windows"] = f"{sample_text()} (oracle: C restatement of the reference path, FP64)"
    out["fp64_evaluations_equal_oracle"] = bool(evals_equal)
    return out


def line_config(n_lines: int, n_wavelengths: int, n_layers: int) -> dict:
    """The ``config`` of a bench line, identical in both arms for one workload."""
    return {"workload": WORKLOAD["name"], "n_lines": int(n_lines), "n_wavelengths": int(n_wavelengths),
            "n_layers": int(n_layers)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cat_path = workload_catalog_path()
    n_full = int(oracle_grid().size)
    for _ in range(max(args.warmup, 0)):
        pass  # the CPU port has no warm-up state; each step is a fresh sample
    res = cpu_baseline(cat_path, steps=max(1, args.steps))
    spectra = (res["points"] / n_full) / res["seconds"]
    line = {
        "impl": "reference", "metric": METRIC, "value": res["evals_per_s"], "unit": "evals/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * res["seconds"] / res["passes"], "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": line_config(WORKLOAD["n_lines"] + WORKLOAD.get("n_band_lines", 0), n_full, 72),
        "precision": "fp64 (the reference's arithmetic)",
        "parallelism": f"{res['threads']} host threads (OpenMP), rank 0 only",
        "spectra_per_s": spectra,
        "spectra_per_s_note": "extrapolated: sample grid points per second / full-grid points",
        "cpu_baseline": {"value": res["evals_per_s"], "unit": "evals/s", "cores": res["threads"],
                         "kind": "port",
                         "sample": f"{sample_text()}, {res['passes']} pass(es) ({res['points']} grid "
                                   f"points, {res['evals']} evaluations) per step"},
        "e2e": {"value": res["evals_per_s"], "unit": "evals/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from kurucz_py_joss_submission_gb300 import _native
    from kurucz_py_joss_submission_gb300.device import (DeviceAtmosphere, DeviceCatalog, DeviceGrid,
                                                         Synthesizer, check_flags, make_options)
    from kurucz_py_joss_submission_gb300.io import atmosphere as atm_io
    from kurucz_py_joss_submission_gb300.io.lines import atomic

    cat_path = workload_catalog_path()
    t = time.time()
    w0, w1 = (args.window if args.window else (WORKLOAD["wl_start"], WORKLOAD["wl_end"]))
    cat = atomic.load_catalog_window(cat_path, w0, w1, sort=True)
    atm = atm_io.load_cached(ROOT / "tests" / "golden" / WORKLOAD["atm"])
    grid = wavelength_grid(w0, w1)
    log(f"catalog {len(cat)} lines, grid {grid.size} points, setup {time.time() - t:.1f}s")
    dcat, datm, dgrid = DeviceCatalog(cat, dev), DeviceAtmosphere(atm, dev), DeviceGrid(grid, device=dev)
    opt = make_options(precision=args.precision, tile_bins=args.tile_bins,
                       warps_per_tile=args.warps_per_tile)
    shard = None
    if world > 1:
        # one spectrum over `world` GPUs: layer blocks -> all-to-all -> wavelength slices
        from kurucz_py_joss_submission_gb300 import sharding

        shard = sharding.ShardRank(dcat, atm, grid, None, rank, world, opt, device=dev)
        st = shard.run(stats=True)
        step = shard.run
        outputs = (shard.flux_total, shard.flux_cont)
    else:
        syn = Synthesizer(dcat, datm, dgrid, opt, keep_asynth=False)
        st = syn.run(stats=True)
        step = syn.run
        outputs = (syn.flux_total, syn.flux_cont)
    evals = st["evaluations"]          # one whole spectrum (summed over ranks)
    launches = st["kernel_launches"]   # this rank's
    log(f"stats {st}")

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # Small workloads fit in L2 (129 MB): flush it (write 256 MB) before every
    # timed step, outside the timed interval; the large ones stream more than
    # L2 per step by themselves.
    small = WORKLOAD["n_lines"] + WORKLOAD.get("n_band_lines", 0) < 200_000 or args.window is not None
    flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device=dev) if small else None
    with ClockSampler(local) as clk:
        barrier()
        if flush_buf is None:
            e0.record()
            for _ in range(args.steps):
                step()
            e1.record()
            barrier()
            ms = e0.elapsed_time(e1)
        else:
            ms = 0.0
            for _ in range(args.steps):
                flush_buf.fill_(1)
                e0.record()
                step()
                e1.record()
                e1.synchronize()
                ms += e0.elapsed_time(e1)
            barrier()
    if world > 1:
        tt = torch.tensor([ms], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
    ms_step = ms / args.steps
    value = evals * args.steps / (ms / 1e3)
    spectra = args.steps / (ms / 1e3)

    # per-stage device times (CUDA events inside the library), for the roofline
    # (N > 1: this rank's opacity half, i.e. its block of layers)
    popt = make_options(precision=args.precision, tile_bins=args.tile_bins,
                        warps_per_tile=args.warps_per_tile, profile=True)
    if shard is not None:
        prof = sharding.ShardRank(dcat, atm, grid, None, rank, world, popt, device=dev)
        prof_run = lambda: prof.opacity(stats=True)
    else:
        prof = Synthesizer(dcat, datm, dgrid, popt, keep_asynth=False)
        prof_run = lambda: prof.run(stats=True)
    stage = {k: [] for k in ("accumulate", "transfer", "pair_setup", "continuum", "partition", "bins_prep", "total")}
    prof_stats = None
    for _ in range(max(3, min(args.steps, 5))):
        prof_stats = prof_run()
        for k in stage:
            stage[k].append(prof_stats["stage_ms"][k])
    stage_ms = {k: statistics.median(v) for k, v in stage.items()}
    del prof

    # end to end: pinned host inputs -> H2D -> synthesis -> D2H of both fluxes,
    # every step.  One GPU: two device input sets, so the copies of step i+1
    # (on a copy stream) overlap the synthesis of step i, as a serving loop
    # would run it; each set is rewritten only after its previous synthesis
    # and D2H have finished.
    def device_inputs(c, a, g):
        return list(c.t.values()) + list(a.t.values()) + [g.wavelength]

    if shard is not None:
        dev_inputs = list(dcat.t.values()) + list(shard.atm_block.t.values()) + list(shard.atm_full.t.values())
        dev_inputs += [shard.grid.wavelength, shard.grid_slice.wavelength]
        sets = [(dev_inputs, step, outputs)]
    else:
        dcat2, datm2, dgrid2 = DeviceCatalog(cat, dev), DeviceAtmosphere(atm, dev), DeviceGrid(grid, device=dev)
        syn2 = Synthesizer(dcat2, datm2, dgrid2, opt, keep_asynth=False)
        syn2.run()
        sets = [(device_inputs(dcat, datm, dgrid), step, outputs),
                (device_inputs(dcat2, datm2, dgrid2), syn2.run, (syn2.flux_total, syn2.flux_cont))]
    host = []
    h2d = 0
    for tns in sets[0][0]:
        hp = torch.empty(tns.shape, dtype=tns.dtype, pin_memory=True)
        hp.copy_(tns.cpu())
        host.append(hp)
        h2d += hp.numel() * hp.element_size()
    outs = [(torch.empty(o[0].numel(), dtype=torch.float64, pin_memory=True),
             torch.empty(o[1].numel(), dtype=torch.float64, pin_memory=True)) for _, _, o in sets]
    d2h = 2 * outputs[0].numel() * 8
    e2e_steps = max(1, min(args.steps, 5))
    main = torch.cuda.current_stream()
    copy_stream = torch.cuda.Stream() if len(sets) > 1 else main
    done = [torch.cuda.Event() for _ in sets]
    ready = [torch.cuda.Event() for _ in sets]
    barrier()
    e0.record()
    for k in range(len(sets)):
        done[k].record(main)
    for i in range(e2e_steps):
        k = i % len(sets)
        dev_in, run_k, out_k = sets[k]
        with torch.cuda.stream(copy_stream):
            copy_stream.wait_event(done[k])
            for hp, tns in zip(host, dev_in):
                tns.copy_(hp, non_blocking=True)
            ready[k].record(copy_stream)
        main.wait_event(ready[k])
        run_k()
        outs[k][0].copy_(out_k[0], non_blocking=True)
        outs[k][1].copy_(out_k[1], non_blocking=True)
        done[k].record(main)
    e1.record()
    barrier()
    e2e_ms = e0.elapsed_time(e1) / e2e_steps
    # every timed step's device flags (sticky on the device): raises if any
    # synthesis above hit an internal limit
    check_flags()
    if world > 1:
        v = torch.tensor([e2e_ms, float(h2d), float(d2h)], dtype=torch.float64, device=dev)
        mx = v[:1].clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        dist.all_reduce(v)
        e2e_ms, h2d, d2h = float(mx.item()), float(v[1].item()), float(v[2].item())
    e2e_value = evals / (e2e_ms / 1e3)

    line = None
    if rank == 0:
        # accuracy of this precision against the all-FP64 path on the same inputs
        ft = outputs[0].cpu().numpy().copy()
        fc = outputs[1].cpu().numpy().copy()
        err = None
        if args.precision != "fp64" and not args.skip_fp64_check and world == 1:
            ref = Synthesizer(dcat, datm, dgrid, make_options(precision="fp64"), keep_asynth=False)
            ref.run()
            torch.cuda.synchronize()
            ft64 = ref.flux_total.cpu().numpy()
            fc64 = ref.flux_cont.cpu().numpy()
            err = flux_errors(ft, fc, ft64, fc64)
            del ref
        hbm_peak, peak_kind = measured_peaks()
        acc_ms = stage_ms["accumulate"]
        L = atm.layers
        # descriptors + positions in, ASYNTH out (N > 1: rank 0's block of layers)
        acc_pairs = prof_stats["valid_pairs"] if shard is not None else st["valid_pairs"]
        acc_layers = (shard.depth_blocks[0][1] - shard.depth_blocks[0][0]) if shard is not None else L
        acc_bytes = acc_pairs * 36.0 + acc_layers * grid.size * 4.0
        acc_evals = prof_stats["evaluations"] if shard is not None else evals
        achieved_gbs = acc_bytes / (acc_ms / 1e3) / 1e9
        traffic = ncu_traffic()
        fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12
        cpu = cpu_baseline(cat_path) if (not args.skip_cpu and world == 1) else None
        vs_port = (accuracy_vs_port(cat_path, datm, cpu, dev)
                   if cpu is not None and not args.skip_fp64_check and args.window is None else None)
        line = {
            "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
            "dtype": "fp32" if args.precision == "mixed" else "f64", "data": "synthetic",
            "config": line_config(len(cat), grid.size, L),
            "precision": args.precision,
            "window": [w0, w1] if args.window else None,
            "l2": ("L2 flushed (256 MB written) before every timed step" if flush_buf is not None
                   else f"inputs larger than L2 (pair descriptors {st['valid_pairs'] * 32 / 1e9:.1f} GB, "
                        f"opacity cubes {3 * L * grid.size * 4 / 1e9:.2f} GB per step)"),
            "parallelism": "1 GPU" if world == 1 else
                           f"{world} GPUs: layer blocks, one all-to-all, wavelength slices",
            "spectra_per_s": spectra,
            "evaluations_per_step": evals,
            "valid_pairs": st["valid_pairs"],
            "stage_ms": stage_ms,
            "accuracy_vs_fp64": err,
            "accuracy_vs_port": vs_port,
            "e2e": {"value": e2e_value, "unit": "evals/s", "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches * args.steps),
            "clocks": clk.summary(),
            "roofline": {"bound": "hbm", "kernel": "accumulate_kernel", "achieved": achieved_gbs,
                         "peak": hbm_peak, "unit": "GB/s", "frac": achieved_gbs / hbm_peak,
                         "peak_kind": peak_kind, "traffic": traffic,
                         "algorithmic_bytes_per_launch": acc_bytes},
            "roofline_fp32": {"kernel": "accumulate_kernel",
                              "achieved": acc_evals * FLOPS_PER_EVAL / (acc_ms / 1e3) / 1e12,
                              "peak": fp32_peak, "unit": "TFLOP/s",
                              "frac": acc_evals * FLOPS_PER_EVAL / (acc_ms / 1e3) / 1e12 / fp32_peak,
                              "peak_kind": "nominal (152 SM x 128 lanes x 2 x 2.07 GHz)"},
        }
        line["cpu_baseline"] = None  # timed on rank 0 at N = 1 only
        if cpu is not None:
            line["cpu_baseline"] = {"value": cpu["evals_per_s"], "unit": "evals/s", "cores": cpu["threads"],
                                    "kind": "port",
                                    "sample": f"{sample_text()}, {cpu['passes']} pass(es) ({cpu['points']} "
                                              f"points, {cpu['evals']} evaluations, {cpu['seconds']:.1f} s)"}
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    if line is not None and world == 1 and not args.no_forms and args.window is None \
            and WORKLOAD["name"] == "full_300_1800":
        line["forms"] = run_forms()
    if line is not None:
        print(json.dumps(line), flush=True)
    return 0


# The other forms of the path, each measured by a child run of this script
# (its own process: memory freed in between, a failure recorded without
# losing the headline): few steps, every timing rule as for the headline.
FORMS = {
    "batch_256": ["--workload", "batch_256", "--steps", "3", "--warmup", "3"],
    "dense_10m": ["--workload", "dense_10m", "--steps", "3", "--warmup", "3", "--skip-cpu"],
    "diff_400_700": ["--workload", "diff_400_700", "--steps", "3", "--warmup", "3", "--fd-params", "40"],
    "pops_256": ["--workload", "pops_256", "--steps", "5", "--warmup", "3"],
    "special_480_520": ["--workload", "special_480_520", "--steps", "5", "--warmup", "3"],
}


def run_forms() -> dict:
    out = {}
    for name, extra in FORMS.items():
        t = time.time()
        try:
            r = subprocess.run([sys.executable, str(ROOT / "bench.py"), *extra, "--no-forms"], cwd=ROOT,
                               capture_output=True, text=True, timeout=900)
            lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
            if r.returncode != 0 or not lines:
                out[name] = {"error": f"rc={r.returncode}: {r.stderr.strip().splitlines()[-1:]}"}
            else:
                out[name] = json.loads(lines[-1])
        except Exception as e:  # noqa: BLE001 -- a form's failure must not lose the headline line
            out[name] = {"error": repr(e)}
        out[name]["wall_s"] = round(time.time() - t, 1)
        log(f"form {name}: {out[name].get('value')} {out[name].get('unit')} ({out[name]['wall_s']} s)")
    return out


def batch_jobs(n_atm: int):
    from kurucz_py_joss_submission_gb300.batch import Job

    rng = np.random.default_rng(BATCH_SEED)
    jobs = []
    for _ in range(BATCH_JOBS):
        a = int(rng.integers(n_atm))
        width = float(rng.uniform(1.0, 50.0))
        start = float(rng.uniform(300.0, 1800.0 - width))
        jobs.append(Job(a, start, start + width))
    return jobs


def run_batch(args):
    """256 syntheses (uneven layer counts and windows, shared 1.5M lines) as
    one captured CUDA graph per step; spectra/s and evaluations/s."""
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from kurucz_py_joss_submission_gb300 import autotune
    from kurucz_py_joss_submission_gb300.batch import BatchSynthesizer
    from kurucz_py_joss_submission_gb300.device import DeviceCatalog, check_flags
    from kurucz_py_joss_submission_gb300.io import atmosphere as atm_io
    from kurucz_py_joss_submission_gb300.io.lines import atomic

    global WORKLOAD
    WORKLOAD = workload_spec("full_300_1800")
    cat = atomic.load_catalog_window(workload_catalog_path(), 300.0, 1800.0, sort=True)
    man = json.loads((ROOT / "tests" / "golden" / "batch_atmospheres.json").read_text())
    atms = [atm_io.load_cached(ROOT / "tests" / "golden" / k["file"]) for k in man["kept"]]
    jobs_all = batch_jobs(len(atms))
    jobs = jobs_all[rank::world]          # jobs are independent: shard them across ranks
    dcat = DeviceCatalog(cat, dev)

    def make(options, workspace):
        o = dict(options)
        groups = o.pop("groups", 1)
        return BatchSynthesizer(dcat, atms, jobs, precision=args.precision, options=o, groups=groups,
                                workspace=workspace, device=dev)

    tuned = autotune.tune(make, autotune.signature(jobs, len(cat), [a.layers for a in atms]), args.precision,
                          log=log)
    bs = make(tuned, None)
    evals = bs.evaluations()
    # stage times of the plan (CUDA events between its launches), medians of 3
    prof = make(dict(tuned, profile=True), bs.workspace)
    stage_runs = [prof.run(stats=True)["stage_ms"] for _ in range(3)]
    stage_ms = {k: statistics.median(r[k] for r in stage_runs) for k in stage_runs[0]}
    del prof
    bs = make(tuned, bs.workspace)
    bs.capture()
    for _ in range(args.warmup):
        bs.replay()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record()
        for _ in range(args.steps):
            bs.replay()
        e1.record()
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    tot = torch.tensor([ms, float(evals), float(len(jobs))], dtype=torch.float64, device=dev)
    if world > 1:
        mx = tot[:1].clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        dist.all_reduce(tot)
        ms, evals = float(mx.item()), int(tot[1].item())
    ms_step = ms / args.steps
    # end to end: pinned host copies of the shared lines, atmospheres and grids in, fluxes out
    host, h2d = [], 0
    dev_in = list(dcat.t.values()) + [t for a in bs.atm for t in a.t.values()] + [g.wavelength for g in bs.grids]
    for t in dev_in:
        hp = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        hp.copy_(t.cpu())
        host.append((hp, t))
        h2d += hp.numel() * hp.element_size()
    outs = [(torch.empty(f.numel(), dtype=torch.float64, pin_memory=True), f) for f in bs.flux_total + bs.flux_cont]
    d2h = sum(o.numel() * 8 for o, _ in outs)
    e2e_steps = max(1, min(args.steps, 5))
    torch.cuda.synchronize()
    e0.record()
    for _ in range(e2e_steps):
        for hp, t in host:
            t.copy_(hp, non_blocking=True)
        bs.replay()
        for o, f in outs:
            o.copy_(f, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / e2e_steps
    check_flags()
    line = None
    if rank == 0:
        err = None
        if args.precision != "fp64" and not args.skip_fp64_check:
            # every job against an all-FP64 single synthesis of its window
            from kurucz_py_joss_submission_gb300.device import DeviceAtmosphere, DeviceGrid, Synthesizer, make_options

            per = []
            datm = [DeviceAtmosphere(a, device=dev) for a in atms]
            for i, j in enumerate(jobs):
                rows = bs.rows[i]
                sub = DeviceCatalog(cat.take(np.arange(rows.start, rows.stop)), dev)
                ref = Synthesizer(sub, datm[j.atmosphere], bs.grids[i], make_options(precision="fp64"),
                                  keep_asynth=False)
                ref.run()
                ft, fc = bs.flux_total[i].cpu().numpy(), bs.flux_cont[i].cpu().numpy()
                per.append(flux_errors(ft, fc, ref.flux_total.cpu().numpy(), ref.flux_cont.cpu().numpy()))
                del ref, sub
            err = merge_errors(per)
            err["norm_flux_max_rel_median_spectrum"] = float(np.median([p["norm_flux_max_rel"] for p in per]))
            err["spectra_checked"] = len(per)
        npts = [g.n for g in bs.grids]
        line = {
            "metric": "spectra/s (batched: 256 atmospheres x windows, one batch plan = 15 persistent launches, "
                      "replayed as a CUDA graph per step)",
            "value": len(jobs_all) * args.steps / (ms / 1e3), "unit": "spectra/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
            "dtype": "fp32" if args.precision == "mixed" else "f64", "data": "synthetic",
            "config": {"workload": "batch_256", "jobs": len(jobs_all), "atmospheres": len(atms),
                       "layers": sorted({a.layers for a in atms}), "grid_points_min": int(min(npts)),
                       "grid_points_max": int(max(npts)), "grid_points_total": int(sum(npts)),
                       "n_lines_shared": len(cat), "tuned": tuned, "precision": args.precision,
                       "workspace_bytes": int(bs.workspace_bytes),
                       "l2": "inputs larger than L2 (shared lines 111 MB + per-job descriptors)",
                       "parallelism": "1 GPU" if world == 1 else f"{world} GPUs, jobs split across ranks"},
            "evaluations_per_s": evals * args.steps / (ms / 1e3),
            "evaluations_per_step": evals,
            "stage_ms": stage_ms,
            "accuracy_vs_fp64": err,
            "e2e": {"value": len(jobs_all) / (e2e_ms / 1e3), "unit": "spectra/s", "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "clocks": clk.summary(),
            "roofline": None,
            "cpu_baseline": None,
        }
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    if line is not None:
        print(json.dumps(line), flush=True)
    return 0


POPS_SEED = 404
POPS_MODELS = 256


def pops_models(work: Path) -> list:
    """256 seeded grey ATLAS models with the batched workload's distributions:
    layers uniform in 64..80, Teff log-uniform in 3500..40000 K, log g uniform
    in 0..5, [M/H] uniform in -2..+0.5; written as .atm files."""
    from kurucz_py_joss_submission_gb300 import workloads

    rng = np.random.default_rng(POPS_SEED)
    out = []
    for k in range(POPS_MODELS):
        n = int(rng.integers(64, 81))
        teff = float(math.exp(rng.uniform(math.log(3500.0), math.log(40000.0))))
        logg = float(rng.uniform(0.0, 5.0))
        mh = float(rng.uniform(-2.0, 0.5))
        p = work / f"model_{k}.atm"
        workloads.grey_atmosphere_atm(p, teff, logg, mh, n_layers=n)
        out.append((p, dict(n_layers=n, teff=teff, logg=logg, metallicity=mh)))
    return out


def run_pops(args):
    """FP64 populations (molecular equilibrium, Saha ion populations, Doppler
    widths) of 256 fresh model atmospheres in one ks_populations call per
    step; atmospheres/s, accuracy against the oracle on a sample."""
    import tempfile

    import torch

    from kurucz_py_joss_submission_gb300.physics import populations as P
    from oracle import pops as opops

    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if rank != 0:
        return 0  # one call holds every model; replicas only
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    with tempfile.TemporaryDirectory(prefix="kgb300_pops_") as tmp:
        models = pops_models(Path(tmp))
        parsed = [P.parse_atm_file(p) for p, _ in models]
        dp = P.DevicePopulations(parsed, device=dev)
        for _ in range(args.warmup):
            dp.run()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            e0.record()
            for _ in range(args.steps):
                dp.run()
            e1.record()
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        # end to end: the models' columns in from pinned host memory, every field out
        ins = [(torch.empty(t.shape, dtype=t.dtype, pin_memory=True).copy_(t.cpu()), t)
               for d in dp.inputs for t in d.values()]
        outs = [(torch.empty(t.shape, dtype=t.dtype, pin_memory=True), t) for d in dp.outputs for t in d.values()]
        h2d = sum(h.numel() * h.element_size() for h, _ in ins)
        d2h = sum(h.numel() * h.element_size() for h, _ in outs)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            for h, t in ins:
                t.copy_(h, non_blocking=True)
            dp.run()
            for h, t in outs:
                h.copy_(t, non_blocking=True)
        e1.record()
        torch.cuda.synchronize()
        e2e_ms = e0.elapsed_time(e1) / args.steps
        # accuracy and CPU baseline: the oracle (FP64 restatement, one core) on a sample
        sample = [0, 1, 2, 3, 64, 128, 192, 255]
        mol = {int(c) for c in opops.readmol()[0] if c < 100}
        errs = {"scalars": 0.0, "populations_saha": 0.0, "populations_molecular": 0.0, "doppler": 0.0}
        t0 = time.perf_counter()
        for k in sample:
            ref = opops.convert(models[k][0])
            out = dp.host(k)

            def rel(a, b):
                m = (a != 0) | (b != 0)
                return float(np.max(np.abs(a[m] - b[m]) / np.maximum(np.abs(b[m]), 1e-300))) if m.any() else 0.0

            for f in ("electron_density", "mass_density", "hckt", "xnf_h", "xnf_he1", "xnf_h2"):
                errs["scalars"] = max(errs["scalars"], rel(out[f], ref[f]))
            errs["doppler"] = max(errs["doppler"], rel(out["doppler_per_ion"], ref["doppler_per_ion"]))
            for z in range(1, 100):
                key = "populations_molecular" if z in mol else "populations_saha"
                errs[key] = max(errs[key], rel(out["population_per_ion"][:, :, z - 1],
                                               ref["population_per_ion"][:, :, z - 1]))
        cpu_s = (time.perf_counter() - t0) / len(sample)
        layers = [m[1]["n_layers"] for m in models]
        teffs = [m[1]["teff"] for m in models]
        iters = np.concatenate([dp.host(k)["nmolec_iterations"] for k in range(len(models))])
    line = {
        "metric": "atmospheres/s (FP64 populations: molecular equilibrium, Saha ion populations, Doppler "
                  "widths; 256 models per ks_populations call)",
        "value": POPS_MODELS / (ms / 1e3), "unit": "atmospheres/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "pops_256", "models": POPS_MODELS, "layers": [min(layers), max(layers)],
                   "layers_total": int(sum(layers)), "teff_K": [round(min(teffs)), round(max(teffs))],
                   "seed": POPS_SEED, "l2": "small inputs (~0.2 MB); outputs 245 MB per step, larger than L2",
                   "parallelism": "1 GPU"},
        "newton_iterations": {"total": int(iters.sum()), "max_per_layer": int(iters.max()),
                              "mean_per_layer": float(iters.mean())},
        "accuracy_vs_oracle": dict(errs, models_checked=len(sample)),
        "e2e": {"value": POPS_MODELS / (e2e_ms / 1e3), "unit": "atmospheres/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": 2 * args.steps,
        "clocks": clk.summary(),
        "roofline": None,
        "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "atmospheres/s", "cores": 1, "kind": "port",
                         "sample": f"oracle (FP64 numpy restatement) on {len(sample)} of the models, "
                                   f"{cpu_s:.2f} s per model"},
    }
    print(json.dumps(line), flush=True)
    return 0


SPECIAL = dict(w0=480.0, w1=520.0, n_lines=20000, seed=406, nb_every=100, aut_every=400,
               atm="atm_t5800g444.npz")


def special_catalog_path() -> Path:
    """The 480-520 nm list of the special-lines form: 20,000 seeded metal
    lines, every 100th with NBLO/NBUP (fort.19 NORMAL), every 400th tagged AUT
    (autoionizing), H beta and H gamma, the table's He I lines and three
    merged-continuum (CONTINUU) records."""
    from kurucz_py_joss_submission_gb300 import workloads

    p = Path(os.environ.get("TMPDIR", "/tmp")) / f"kgb300_special_{SPECIAL['seed']}.gf"
    if p.exists():
        return p
    d = workloads.random_atomic_lines(SPECIAL["n_lines"], SPECIAL["w0"] - 0.15, SPECIAL["w1"] + 0.15,
                                      SPECIAL["seed"])
    n = len(d)
    lo, up = np.zeros(n, np.int32), np.zeros(n, np.int32)
    lo[::SPECIAL["nb_every"]], up[::SPECIAL["nb_every"]] = 3, 5
    d.n_lower, d.n_upper = lo, up
    ia = np.arange(SPECIAL["aut_every"] // 2, n, SPECIAL["aut_every"])
    tag = np.array([""] * n, dtype=object)
    tag[ia] = "AUT"
    d.tag = tag
    d.log_gamma_rad[ia], d.log_gamma_vdw[ia] = 11.0, 0.3
    d.log_gamma_stark[ia] = np.where(np.arange(ia.size) % 2 == 0, -0.5, 0.3)
    d.log_gf[ia] = np.minimum(d.log_gf[ia], -1.0) - 12.0
    z = np.zeros(3)
    cont = workloads.LineDraw(wavelength_nm=np.array([485.0, 495.0, 505.0]), log_gf=np.array([-16.0, -15.5, -16.5]),
                              code=np.full(3, 26.00), e_lower_cm=np.full(3, 1500.0), log_gamma_rad=z + 8.0,
                              log_gamma_stark=z - 5.0, log_gamma_vdw=z - 7.5,
                              labelp=np.array(["CONTINUU"] * 3, dtype=object), xjp=np.array([40.0, 50.0, 30.0]))
    d = workloads.merge_lines(d, workloads.balmer_lines([4, 5]), workloads.helium_lines(SPECIAL["w0"], SPECIAL["w1"]),
                              cont)
    tmpname = p.with_suffix(f".{os.getpid()}.tmp")
    workloads.write_gfall(tmpname, d)
    os.replace(tmpname, p)
    return p


def run_special(args):
    """One 480-520 nm synthesis of a list holding every special line class
    (hydrogen, helium, fort.19 NORMAL / autoionizing / merged continuum):
    spectra/s, the special-line stage, the same synthesis without the special
    lines, and the mixed path's error against FP64."""
    import torch

    from kurucz_py_joss_submission_gb300.device import (DeviceAtmosphere, DeviceCatalog, DeviceGrid,
                                                         Synthesizer, make_options)
    from kurucz_py_joss_submission_gb300.io import atmosphere as atm_io
    from kurucz_py_joss_submission_gb300.io.lines import atomic

    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if rank != 0:
        return 0  # one window: replicas only
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w0, w1 = SPECIAL["w0"], SPECIAL["w1"]
    cat = atomic.load_catalog_window(special_catalog_path(), w0, w1, sort=True)
    atm = atm_io.load_cached(ROOT / "tests" / "golden" / SPECIAL["atm"])
    grid = wavelength_grid(w0, w1)
    dcat, datm, dgrid = DeviceCatalog(cat, dev), DeviceAtmosphere(atm, dev), DeviceGrid(grid, device=dev)
    counts = {"hydrogen": dcat.n_hydrogen, "helium": dcat.n_helium, "fort19": dcat.n_f19}
    syn = Synthesizer(dcat, datm, dgrid, make_options(precision="mixed"), keep_asynth=False)
    st = syn.run(stats=True)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)   # inputs fit in L2: flush per step

    def timed(run):
        for _ in range(args.warmup):
            run()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        total = 0.0
        for _ in range(args.steps):
            flush.fill_(1)
            e0.record()
            run()
            e1.record()
            e1.synchronize()
            total += e0.elapsed_time(e1)
        return total / args.steps

    with ClockSampler(local) as clk:
        ms = timed(syn.run)
    rec = dcat.rec
    saved = (rec.n_hydrogen, rec.n_helium, rec.n_f19)
    rec.n_hydrogen = rec.n_helium = rec.n_f19 = 0
    ms_plain = timed(syn.run)
    rec.n_hydrogen, rec.n_helium, rec.n_f19 = saved
    syn.run()   # the fluxes compared below: with the special lines again
    prof = Synthesizer(dcat, datm, dgrid, make_options(precision="mixed", profile=True), keep_asynth=False)
    stages = [prof.run(stats=True)["stage_ms"] for _ in range(5)]
    stage_ms = {k: statistics.median(s[k] for s in stages) for k in stages[0]}
    ft, fc = syn.flux_total.cpu().numpy(), syn.flux_cont.cpu().numpy()
    ref = Synthesizer(dcat, datm, dgrid, make_options(precision="fp64"), keep_asynth=False)
    ref.run()
    torch.cuda.synchronize()
    err = flux_errors(ft, fc, ref.flux_total.cpu().numpy(), ref.flux_cont.cpu().numpy())
    line = {
        "metric": "spectra/s (480-520 nm, 20,000 lines with hydrogen, helium and fort.19 lines, mixed)",
        "value": 1e3 / ms, "unit": "spectra/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
        "dtype": "fp32", "data": "synthetic",
        "config": {"workload": "special_480_520", "grid_points": int(grid.size), "lines": len(cat),
                   "special_lines": counts, "atmosphere": SPECIAL["atm"], "seed": SPECIAL["seed"],
                   "l2": "inputs smaller than L2: 256 MB written before every timed step",
                   "parallelism": "1 GPU"},
        "ms_without_special_lines": ms_plain,
        "stage_ms": stage_ms,
        "evaluations_per_step": int(st["evaluations"]),
        "accuracy_vs_fp64": err,
        "gpu_launches": int(st["kernel_launches"]) * args.steps,
        "clocks": clk.summary(),
        "roofline": None,
        "cpu_baseline": None,
    }
    print(json.dumps(line), flush=True)
    return 0


DIFF_ELEMENTS = (1, 2, 6, 7, 8, 11, 12, 13, 14, 16, 19, 20, 22, 23, 24, 25, 26, 27, 28, 29)


def run_diff(args):
    """Differentiable synthesis (400-700 nm, 500k lines, Teff 6000 K log g 4.3,
    the atmosphere recomputed from its .atm model on the GPU for every
    evaluation): loss = sum (F/Fc - target)^2 with the target synthesised
    from log gf offsets ~ N(0, 0.1) and offsets ~ N(0, 0.05) dex of 20 element
    abundances; one step = forward + adjoint (gradients for 4 x 500k line
    parameters and the 20 log abundances).  Central finite differences
    (h = 1e-4 dex) on --fd-params line parameters, half the most sensitive
    lines of each class and half at random, and on every abundance (with h
    reduced to 1e-5 / 1e-6 dex where the two runs cross a gate or wing-reach
    step, which the adjoint holds fixed), check the gradient."""
    import torch

    from kurucz_py_joss_submission_gb300 import autodiff, workloads
    from kurucz_py_joss_submission_gb300.io import atmosphere as atm_io
    from kurucz_py_joss_submission_gb300.io.lines import atomic

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    w0, w1, n_lines, seed = 400.0, 700.0, 500_000, 20245
    p = Path(os.environ.get("TMPDIR", "/tmp")) / f"kgb300_diff_{seed}.gf"
    if not p.exists():
        d = workloads.random_atomic_lines(n_lines, w0 - 1.0, w1 + 1.0, seed)
        tmp = p.with_suffix(f".{os.getpid()}.tmp")
        workloads.write_gfall(tmp, d)
        os.replace(tmp, p)
    cat = atomic.load_catalog_window(p, w0, w1, sort=True)
    atm = atm_io.load_cached(ROOT / "tests" / "golden" / "atm_t6000g430.npz")
    global WORKLOAD
    WORKLOAD = dict(workload_spec("full_300_1800"), wl_start=w0, wl_end=w1)
    grid = wavelength_grid(w0, w1)
    ds = autodiff.AtmosphereDiffSynthesizer(cat, ROOT / "tests" / "golden" / "atm_t6000g430.atm", atm, grid,
                                            DIFF_ELEMENTS, device=dev)
    n = len(cat)
    ne = len(DIFF_ELEMENTS)
    rng = np.random.default_rng(seed + 1)
    pert = torch.tensor(rng.normal(0.0, 0.1, n), dtype=torch.float64, device=dev)
    pert_ab = torch.tensor(rng.normal(0.0, 0.05, ne), dtype=torch.float64, device=dev)
    ft, fc = ds.forward(pert, None, None, None, pert_ab)
    target = (ft / fc).clone()
    zeros = [torch.zeros(n, dtype=torch.float64, device=dev) for _ in range(4)]
    zeros_ab = torch.zeros(ne, dtype=torch.float64, device=dev)

    def step():
        ps = [z.clone().requires_grad_(True) for z in zeros] + [zeros_ab.clone().requires_grad_(True)]
        a, b = autodiff.synthesize_atmosphere(ds, *ps)
        loss = torch.sum((a / b - target) ** 2)
        loss.backward()
        return loss, ps

    for _ in range(max(1, args.warmup)):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = max(1, args.steps)
    with ClockSampler(0) as clk:
        e0.record()
        for _ in range(steps):
            loss, ps = step()
        e1.record()
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    grads = [q.grad.cpu().numpy() for q in ps]
    # forward alone, for the split
    e0.record()
    for _ in range(steps):
        ds.forward()
    e1.record()
    torch.cuda.synchronize()
    fwd_ms = e0.elapsed_time(e1) / steps
    fd = None
    if not args.skip_fp64_check:
        h = 1e-4
        names = ("log_gf", "log_gamma_rad", "log_gamma_stark", "log_gamma_vdw")
        errs = {k: [] for k in names}
        # half among the most sensitive lines of each parameter class, half at random
        k = max(1, args.fd_params // 8)
        picks = [(p_, int(i)) for p_ in range(4) for i in np.argsort(-np.abs(grads[p_]))[:k]]
        picks += [(int(rng.integers(4)), int(rng.integers(n))) for _ in range(args.fd_params - len(picks))]
        for par, i in picks:
            vals = []
            for sgn in (+1, -1):
                d = [z.clone() for z in zeros]
                d[par][i] = sgn * h
                a, b = ds.forward(*d)
                vals.append(float(torch.sum((a / b - target) ** 2).item()))
            g_fd = (vals[0] - vals[1]) / (2 * h)
            g_ad = float(grads[par][i])
            scale = max(abs(g_fd), abs(g_ad))
            # compare where the central difference resolves the gradient:
            # a loss change of at least 1e-11 of the loss over +-h
            if scale * h > 1e-11 * max(abs(float(loss.item())), 1e-300):
                errs[names[par]].append(abs(g_fd - g_ad) / scale)
        # abundances: every element, with h shrunk where the +-h runs cross a step
        ab_err, ab_h = [], []
        for i in range(ne):
            for hh in (1e-4, 1e-5, 1e-6):
                vals, counts = [], []
                for sgn in (+1, -1):
                    d = zeros_ab.clone()
                    d[i] = sgn * hh
                    a, b = ds.forward(None, None, None, None, d, stats=True)
                    vals.append(float(torch.sum((a / b - target) ** 2).item()))
                    counts.append((ds.last_stats["valid_pairs"], ds.last_stats["evaluations"]))
                if counts[0] == counts[1]:
                    break
            else:
                continue
            g_fd = (vals[0] - vals[1]) / (2 * hh)
            g_ad = float(grads[4][i])
            scale = max(abs(g_fd), abs(g_ad))
            if scale * hh > 1e-11 * max(abs(float(loss.item())), 1e-300):
                ab_err.append(abs(g_fd - g_ad) / scale)
                ab_h.append(hh)
        errs["log_abundance"] = ab_err
        allerr = np.array([e for v in errs.values() for e in v])
        fd = {"params_checked": args.fd_params, "params_resolved_by_fd": int(allerr.size), "h_dex": h,
              "rel_err_median": float(np.median(allerr)) if allerr.size else None,
              "rel_err_p90": float(np.percentile(allerr, 90)) if allerr.size else None,
              "frac_within_5pct": float(np.mean(allerr < 0.05)) if allerr.size else None,
              "by_parameter": {k: {"n": len(v), "rel_err_median": float(np.median(v)) if v else None,
                                   "frac_within_5pct": float(np.mean(np.array(v) < 0.05)) if v else None}
                               for k, v in errs.items()},
              "abundance_h_dex": ab_h,
              "abundance_rel_err_max": float(np.max(ab_err)) if ab_err else None}
    line = {
        "metric": "forward+adjoint steps/s (differentiable synthesis: d loss / d log gf and 3 log damping "
                  "constants for every line, and 20 log abundances)",
        "value": 1e3 / ms, "unit": "steps/s", "n_gpus": 1, "steps": steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": "diff_400_700", "n_lines": n, "n_wavelengths": int(grid.size), "n_layers": atm.layers,
                   "parameters": 4 * n + ne, "atmosphere": "Teff 6000 K, log g 4.30 (.atm; populations on the GPU "
                   "every evaluation, continuum tables from its converted model)",
                   "abundances": list(DIFF_ELEMENTS),
                   "target": "log gf offsets ~ N(0, 0.1) and 20 abundance offsets ~ N(0, 0.05) dex (per-layer T "
                             "offsets: not covered, the continuum opacity stage is not on the GPU)",
                   "l2": "inputs larger than L2 (FP64 descriptors ~1 GB)"},
        "forward_ms": fwd_ms, "adjoint_ms": ms - fwd_ms,
        "loss": float(loss.item()), "skipped_wavelengths_maxj": ds.skipped,
        "finite_difference_check": fd, "clocks": clk.summary(),
        "roofline": None, "cpu_baseline": None, "gpu_launches": None,
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--tile-bins", type=int, default=0)
    ap.add_argument("--warps-per-tile", type=int, default=0)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-fp64-check", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="headline workload only: do not measure the batched, dense and differentiable forms")
    ap.add_argument("--fd-params", type=int, default=200,
                    help="diff_400_700: parameters checked by central finite differences")
    ap.add_argument("--window", type=float, nargs=2, default=None,
                    help="restrict the workload to a wavelength window (small profiling case)")
    ap.add_argument("--workload", choices=sorted(BENCH_WORKLOADS) + ["batch_256", "diff_400_700", "pops_256",
                                                                     "special_480_520"],
                    default="full_300_1800",
                    help="full_300_1800 (headline: 1.5M lines, Teff 5800 K), window_500_510 (20k lines, "
                         "the CPU-runnable reference case), dense_10m (10M lines, Teff 2500 K, log g -1)")
    args = ap.parse_args()
    global WORKLOAD
    if args.workload == "diff_400_700":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no gradients"}))
            return 0
        return run_diff(args)
    if args.workload == "pops_256":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "population workload: timed on the GPU path only"}))
            return 0
        return run_pops(args)
    if args.workload == "special_480_520":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "special-lines workload: timed on the GPU path only"}))
            return 0
        return run_special(args)
    if args.workload == "batch_256":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "batched workload: timed on the GPU path only"}))
            return 0
        return run_batch(args)
    WORKLOAD = workload_spec(args.workload)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    raise SystemExit(main())
