"""Command-line entry point with the reference's flags (synthe_py/cli.py:15-154).

``python -m kurucz_py_joss_submission_gb300.cli MODEL.atm LINES.gf --npz X.npz
--spec out.spec --wl-start A --wl-end B`` behaves like ``python -m
synthe_py.cli`` for the plain-line LTE path; --precision/--tile-bins/
--warps-per-tile select the GPU arithmetic and tiling.
"""

from __future__ import annotations

import argparse
import logging
from pathlib import Path
from typing import Optional

from . import config
from .engine.opacity import run_synthesis


def build_parser() -> argparse.ArgumentParser:
    p = argparse.ArgumentParser(description="GB300 SYNTHE line-opacity and transfer synthesis")
    p.add_argument("model", type=Path, help="model atmosphere: an ATLAS .atm deck or its converted .npz")
    p.add_argument("atomic", type=Path, help="line list in gfall fixed-width format")
    p.add_argument("--npz", type=Path, default=None, help="converted atmosphere to read instead of MODEL")
    p.add_argument("--spec", type=Path, default=Path("spectrum.spec"), help="where to write the three-column .spec")
    p.add_argument("--wl-start", type=float, default=300.0, help="first wavelength of the grid, nm")
    p.add_argument("--wl-end", type=float, default=1800.0, help="last wavelength of the grid, nm")
    p.add_argument("--resolution", type=float, default=300_000.0, help="lambda / delta-lambda of the log grid")
    p.add_argument("--no-vacuum", action="store_true", help="line wavelengths are in air, not vacuum")
    p.add_argument("--cutoff", type=float, default=1e-3, help="KAPMIN as a fraction of the continuum")
    p.add_argument("--linout", type=int, default=30, help="LINOUT switch of SYNTHE")
    p.add_argument("--cache", type=Path, default=None,
                   help="line cache directory of the reference; not used here (the native reader parses "
                        "1.5M lines in well under a second), a warning is logged")
    p.add_argument("--allow-tfort-runtime", action="store_true", help="Accepted, unused")
    p.add_argument("--n-workers", type=int, default=None,
                   help="host worker threads of the reference; not used (the path runs on the GPU), "
                        "a warning is logged")
    p.add_argument("--nlte", action="store_true",
                   help="NLTE line source of the reference: not supported (LTE only), rejected")
    p.add_argument("--scat-iterations", type=int, default=8)
    p.add_argument("--scat-tol", type=float, default=1e-3)
    p.add_argument("--rhoxj", type=float, default=0.0, help="RHOXJ of the line scattering fraction (0: none)")
    p.add_argument("--log-level", type=str, default="INFO",
                   choices=["DEBUG", "INFO", "WARNING", "ERROR"])
    p.add_argument("--diagnostics", type=Path, default=None)
    p.add_argument("--microturb", type=float, default=0.0, help="extra microturbulent velocity, km/s")
    p.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    p.add_argument("--tile-bins", type=int, default=0)
    p.add_argument("--warps-per-tile", type=int, default=0)
    p.add_argument("--populations", choices=["npz", "gpu"], default="npz",
                   help="npz: populations from the converted model; gpu: recomputed from MODEL.atm on the GPU "
                        "in FP64 (molecular equilibrium, Saha, Doppler), continuum tables from the .npz")
    return p


log = logging.getLogger(__name__)


def main(argv: Optional[list] = None) -> int:
    parser = build_parser()
    args = parser.parse_args(argv)
    if args.nlte:
        # the reference's --nlte switches the line source to departure
        # coefficients (physics/bfudge_tables.py); this path computes the
        # LTE source only, so running would give a different spectrum
        parser.error("--nlte is not supported: this GPU path computes the LTE line source only")
    cfg = config.SynthesisConfig.from_cli(
        spec_path=args.spec, diagnostics_path=args.diagnostics, atmosphere_path=args.model,
        atomic_catalog=args.atomic, wl_start=args.wl_start, wl_end=args.wl_end,
        resolution=args.resolution, velocity_microturb=args.microturb,
        vacuum=not args.no_vacuum, cutoff=args.cutoff, linout=args.linout, nlte=args.nlte,
        scattering_iterations=args.scat_iterations, scattering_tolerance=args.scat_tol,
        rhoxj_scale=args.rhoxj, npz_path=args.npz, n_workers=args.n_workers,
        allow_tfort_runtime=args.allow_tfort_runtime, precision=args.precision,
        tile_bins=args.tile_bins, warps_per_tile=args.warps_per_tile,
        populations=args.populations,
    )
    cfg.log_level = args.log_level
    logging.basicConfig(level=getattr(logging, args.log_level),
                        format="%(asctime)s [%(levelname)s] %(name)s - %(message)s")
    if args.cache is not None:
        log.warning("--cache %s ignored: line lists are parsed by the native reader on every run", args.cache)
    if args.n_workers is not None:
        log.warning("--n-workers %d ignored: the synthesis runs on the GPU", args.n_workers)
    run_synthesis(cfg)
    return 0


if __name__ == "__main__":  # pragma: no cover
    raise SystemExit(main())
