"""Generate the golden fixtures by running the reference pipeline itself.

Test infrastructure, run in a container that has the reference checkout
(``--reference DIR`` or ``$SYNTHE_PY_REFERENCE``, default
``/root/reference``; it is never read at test time).  Numba is not
installed there, so ``numba_shim/`` (identity ``jit``, ``prange = range``) is
put first on ``PYTHONPATH`` and the reference executes as plain Python with
NumPy semantics.

For every atmosphere in :data:`ATMOSPHERES` the script writes the ``.atm``
(from :mod:`kurucz_py_joss_submission_gb300.workloads`), converts it with the
reference's own ``synthe_py/tools/convert_atm_to_npz.py`` and keeps the
fields the synthesis path reads (``atm_<name>.npz``).  For every case in
:data:`CASES` it writes the seeded gfall file, runs
``python -m synthe_py.cli`` with ``SYNTHE_PY_STAGE_DUMPS`` and stores the
stage arrays (``case_<name>.npz``): TRANSP + valid mask + centre bins
(stage 3), ASYNTH (stage 4), continuum and fluxes (stage 5), the ``.spec``
columns, and the sha256 of the gfall text so a test can confirm that
regenerating the line list from its seed gives the same file.

Usage: ``python tests/golden/make_golden.py [--reference DIR] [case ...]``
"""

from __future__ import annotations

import hashlib
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
REFERENCE = Path(os.environ.get("SYNTHE_PY_REFERENCE", "/root/reference"))
sys.path.insert(0, str(REPO))

from kurucz_py_joss_submission_gb300 import workloads  # noqa: E402

# Fields of the converted atmosphere that the synthesis path reads
# (synthe_py/io/atmosphere.py:82 load_cached, populations.py:131,
# continuum.py:73).
ATM_FIELDS = (
    "depth", "temperature", "gas_pressure", "electron_density", "mass_density",
    "turbulent_velocity", "hckt", "xnf_h", "xnf_he1", "xnf_h2",
    "population_per_ion", "doppler_per_ion", "wledge", "half_edge",
    "delta_edge", "cont_abs_coeff", "cont_scat_coeff", "cont_coeff_log10",
    "teff", "glog",
)

ATMOSPHERES = {
    "t5800g444": dict(teff=5800.0, logg=4.44, metallicity=0.0),
    "t6000g430": dict(teff=6000.0, logg=4.30, metallicity=0.0),
    "t2500gm10": dict(teff=2500.0, logg=-1.0, metallicity=0.0),
    "t20000g400": dict(teff=20000.0, logg=4.0, metallicity=0.0),
    # t5800g444 with the Doppler widths of Fe and Ti set so that the Voigt
    # table step TABSTEP = 200 / (DOPPLE * RESOLU) is 0.7 (Fe) and 1.1 (Ti):
    # for such steps the reference's incremental TABI (line_opacity.py:540-548)
    # and the closed form 0.5 + n*TABSTEP fall on different sides of an
    # integer at about a hundred offsets of the near wing.  The populations
    # are scaled by the same factor, so XNFDOP = pop / (rho dop) and the
    # TRANSP gates are those of the unmodified atmosphere.
    "t5800g444_tabi": dict(teff=5800.0, logg=4.44, metallicity=0.0, tabstep={26: 0.7, 22: 1.1},
                           tabi_window=(500.0, 501.0)),
}

# name: atmosphere, window, line draw.  Line windows extend 0.15 nm past the
# synthesis window so margin lines (centre outside the grid, wings inside)
# are exercised.
CASES = {
    "tiny_500_501": dict(atm="t5800g444", wl_start=500.0, wl_end=501.0,
                         n_lines=200, draw=(499.85, 501.15), log_uniform=False, seed=11),
    "uv_300_302": dict(atm="t5800g444", wl_start=300.0, wl_end=302.0,
                       n_lines=1500, draw=(299.85, 302.15), log_uniform=False, seed=12),
    "strong_600_601": dict(atm="t6000g430", wl_start=600.0, wl_end=601.0,
                           n_lines=300, draw=(599.85, 601.15), log_uniform=False, seed=13,
                           strong=True),
    "window_500_510": dict(atm="t5800g444", wl_start=500.0, wl_end=510.0,
                           n_lines=20_000, draw=(500.0, 510.0), log_uniform=False, seed=20240),
    # cool giant with molecular-band-like lines (the dense stress case's physics)
    "cool_600_601": dict(atm="t2500gm10", wl_start=600.0, wl_end=601.0,
                         n_lines=200, draw=(599.85, 601.15), log_uniform=False, seed=14,
                         band_lines=800, band_seed=15),
    # line scattering: FSCAT = exp(-RHOX / RHOXJ) splits ASYNTH into
    # absorption and scattering (engine/opacity.py:2408-2440)
    "scat_500_501": dict(atm="t5800g444", wl_start=500.0, wl_end=501.0,
                         n_lines=200, draw=(499.85, 501.15), log_uniform=False, seed=16,
                         rhoxj=0.3),
    # synthesis microturbulence added to the TRANSP Doppler width
    # (physics/line_opacity.py:629)
    "micro_500_501": dict(atm="t5800g444", wl_start=500.0, wl_end=501.0,
                          n_lines=200, draw=(499.85, 501.15), log_uniform=False, seed=17,
                          microturb=2.0),
    # near-wing Voigt table index at rounding ties of TABI (see t5800g444_tabi)
    "tabi_500_501": dict(atm="t5800g444_tabi", wl_start=500.0, wl_end=501.0,
                         n_lines=200, draw=(499.85, 501.15), log_uniform=False, seed=18),
    # hydrogen Balmer lines (HPROF4 profiles, engine/opacity.py:1706): H beta
    # centred in the window (wings of the 2 -> 4 line: the simple-wing branch)
    # and H gamma (2 -> 5: the tapered wings with the m -+ 1, 2 cuts), with
    # H delta beside each, on top of metal lines
    "hbeta_486": dict(atm="t5800g444", wl_start=485.6, wl_end=486.9,
                      n_lines=150, draw=(485.45, 487.05), log_uniform=False, seed=19,
                      hydrogen=[4, 5, 6]),
    "hgamma_434": dict(atm="t5800g444", wl_start=433.5, wl_end=434.8,
                       n_lines=150, draw=(433.35, 434.95), log_uniform=False, seed=20,
                       hydrogen=[4, 5, 6]),
    # helium lines (line types -3 / -6, the helium wing pass of
    # engine/opacity.py:2515-3590 added as AHE x STIM, :3650-3660) in a
    # 20,000 K atmosphere: He I 447.1 nm and He II 468.6 nm on metal lines
    "hei_447": dict(atm="t20000g400", wl_start=446.9, wl_end=447.7,
                    n_lines=120, draw=(446.75, 447.85), log_uniform=False, seed=21,
                    helium=True),
    "heii_468": dict(atm="t20000g400", wl_start=468.3, wl_end=469.1,
                     n_lines=120, draw=(468.15, 469.25), log_uniform=False, seed=22,
                     helium=True),
    # metal lines with NBLO/NBUP set (every 4th line): routed to fort.19 and
    # given _add_fort19_asynth's profiles (engine/opacity.py:1335-1488)
    # instead of TRANSP/ASYNTH's
    "fort19_500_501": dict(atm="t5800g444", wl_start=500.0, wl_end=501.0,
                           n_lines=160, draw=(499.85, 501.15), log_uniform=False, seed=24,
                           nb_every=4),
    # autoionizing lines (gfall AUT tag, every 5th line; ASHORE of both
    # signs): the fort.19 Fano-type profile (engine/opacity.py:901-963)
    "aut_500_501": dict(atm="t5800g444", wl_start=500.0, wl_end=501.0,
                        n_lines=150, draw=(499.85, 501.15), log_uniform=False, seed=25,
                        aut_every=5),
    # merged-continuum records (LABELP CONTINUU, NLAST = XJP): the fort.19
    # ramp between the merge and tail wavelengths (engine/opacity.py:723-758,
    # :863-898), one record below the window
    "cont_505_507": dict(atm="t5800g444", wl_start=505.5, wl_end=507.5,
                         n_lines=120, draw=(505.35, 507.65), log_uniform=False, seed=26,
                         continuum_records=[(505.42, 40.0, -13.0), (505.62, 50.0, -12.5), (506.55, 30.0, -13.5)]),
    # fort.19 continuum-merge limits: Mg I lines with NBLO/NBUP and ISO2 = 2
    # (NCON 2: WCON near 252 nm, WTAIL near 256 nm, per layer) and a He II
    # line with NBLO/NBUP and ISO2 = 5 (WCON near 587 nm, WTAIL near 605 nm)
    "ncon_252": dict(atm="t5800g444", wl_start=251.6, wl_end=253.2,
                     n_lines=80, draw=(251.45, 253.35), log_uniform=False, seed=27,
                     ncon_lines=dict(code=12.00, iso2=2, every=4, nb=(3, 6))),
    "heii_595": dict(atm="t20000g400", wl_start=594.6, wl_end=595.4,
                     n_lines=80, draw=(594.45, 595.55), log_uniform=False, seed=28,
                     ncon_extra=[(595.0, 1.5, 421352.5, 2.01, 5, 24, 5)], helium=True),
}

# Cases too large to commit every stage array for: keep a subset.
LARGE_CASES = {"window_500_510"}


def _env() -> dict:
    env = dict(os.environ)
    env["PYTHONDONTWRITEBYTECODE"] = "1"
    env["PYTHONPATH"] = f"{HERE / 'numba_shim'}:{REFERENCE}"
    return env


def case_lines(case: dict) -> workloads.LineDraw:
    lines = workloads.random_atomic_lines(
        case["n_lines"], case["draw"][0], case["draw"][1], case["seed"],
        log_uniform=case["log_uniform"],
    )
    if case.get("band_lines"):
        bands = workloads.random_band_lines(case["band_lines"], case["draw"][0], case["draw"][1],
                                            case["band_seed"])
        lines = workloads.merge_lines(lines, bands)
    if case.get("hydrogen"):
        lines = workloads.merge_lines(lines, workloads.balmer_lines(case["hydrogen"]))
    if case.get("helium"):
        lines = workloads.merge_lines(lines, workloads.helium_lines(*case["draw"]))
    if case.get("nb_every"):
        k = case["nb_every"]
        lo, up = lines.levels()
        lo, up = lo.copy(), up.copy()
        lo[::k], up[::k] = 3, 5
        lines.n_lower, lines.n_upper = lo, up
        idx = np.arange(0, len(lines), k)
        lines.log_gf[idx] = np.maximum(lines.log_gf[idx], -0.5)   # strong enough to pass the gates
        lines.e_lower_cm[idx] = np.minimum(lines.e_lower_cm[idx], 20000.0)
    if case.get("aut_every"):
        k = case["aut_every"]
        idx = np.arange(0, len(lines), k)
        tag = np.array([""] * len(lines), dtype=object)
        tag[idx] = "AUT"
        lines.tag = tag
        lines.log_gamma_rad[idx] = 11.0
        lines.log_gamma_stark[idx] = np.where(np.arange(idx.size) % 2 == 0, -0.5, 0.3)
        lines.log_gamma_vdw[idx] = 0.3
        lines.log_gf[idx] = np.minimum(lines.log_gf[idx], -1.0) - 12.0
    if case.get("continuum_records"):
        recs = case["continuum_records"]
        z = np.zeros(len(recs))
        extra = workloads.LineDraw(
            wavelength_nm=np.array([r[0] for r in recs]), log_gf=np.array([r[2] for r in recs]),
            code=np.full(len(recs), 26.00), e_lower_cm=np.full(len(recs), 1500.0),
            log_gamma_rad=z + 8.0, log_gamma_stark=z - 5.0, log_gamma_vdw=z - 7.5,
            labelp=np.array(["CONTINUU"] * len(recs), dtype=object), xjp=np.array([r[1] for r in recs]))
        lines = workloads.merge_lines(lines, extra)
    if case.get("ncon_lines"):
        spec = case["ncon_lines"]
        idx = np.arange(0, len(lines), spec["every"])
        lo, up = lines.levels()
        lo, up = lo.copy(), up.copy()
        lo[idx], up[idx] = spec["nb"]
        lines.n_lower, lines.n_upper = lo, up
        iso2 = np.zeros(len(lines), np.int32)
        iso2[idx] = spec["iso2"]
        lines.iso2 = iso2
        lines.code[idx] = spec["code"]
        lines.log_gf[idx] = np.maximum(lines.log_gf[idx], -1.0)
        lines.e_lower_cm[idx] = np.minimum(lines.e_lower_cm[idx], 20000.0)
    if case.get("ncon_extra"):
        recs = case["ncon_extra"]
        z = np.zeros(len(recs))
        extra = workloads.LineDraw(
            wavelength_nm=np.array([r[0] for r in recs]), log_gf=np.array([r[1] for r in recs]),
            code=np.array([r[3] for r in recs]), e_lower_cm=np.array([r[2] for r in recs]),
            log_gamma_rad=z + 8.5, log_gamma_stark=z - 4.0, log_gamma_vdw=z - 7.6,
            n_lower=np.array([r[4] for r in recs], np.int32), n_upper=np.array([r[5] for r in recs], np.int32),
            iso2=np.array([r[6] for r in recs], np.int32))
        lines = workloads.merge_lines(lines, extra)
    if case.get("strong"):
        # push a handful of lines to saturation so the surface optical depth
        # of their cores exceeds the last JOSH tau point (MAXJ = 1 path)
        idx = np.arange(0, len(lines), 25)
        lines.log_gf[idx] = 2.5
        lines.code[idx] = 20.01
        lines.e_lower_cm[idx] = np.minimum(lines.e_lower_cm[idx], 50.0)
    return lines


def build_atmosphere(name: str, work: Path) -> Path:
    spec = ATMOSPHERES[name]
    atm_path = HERE / f"atm_{name}.atm"
    workloads.grey_atmosphere_atm(atm_path, spec["teff"], spec["logg"], spec["metallicity"])
    full_npz = work / f"{name}_full.npz"
    subprocess.run(
        [sys.executable, str(REFERENCE / "synthe_py/tools/convert_atm_to_npz.py"),
         str(atm_path), str(full_npz),
         "--atlas-tables", str(REFERENCE / "synthe_py/data/atlas_tables.npz")],
        check=True, env=_env(), cwd=work, stdout=subprocess.DEVNULL,
    )
    if spec.get("tabstep"):
        # RESOLU = 1 / (ratio - 1) of the window's grid (line_opacity.py:235-239),
        # then a Doppler width whose TABSTEP = 200 * (1 / (DOPPLE * RESOLU)) is
        # the double nearest the chosen step (searched ulp by ulp)
        sys.path.insert(0, str(REPO))
        from oracle import oracle

        grid = oracle.wavelength_grid(*spec["tabi_window"], 300000.0)
        resolu = 1.0 / (grid[1] / grid[0] - 1.0)
        with np.load(full_npz, allow_pickle=False) as d:
            full = {k: np.asarray(d[k]) for k in d.files}
        for z, step in spec["tabstep"].items():
            dop = 200.0 / (step * resolu)
            for _ in range(256):
                ts = 200.0 * (1.0 / (dop * resolu))
                if ts == step:
                    break
                dop = float(np.nextafter(dop, np.inf if ts > step else -np.inf))
            scale = dop / full["doppler_per_ion"][:, :, z - 1]
            full["doppler_per_ion"][:, :, z - 1] = dop
            full["population_per_ion"][:, :, z - 1] *= scale
        np.savez(full_npz, **full)
    with np.load(full_npz) as d:
        kept = {k: np.asarray(d[k]) for k in ATM_FIELDS if k in d}
    out = HERE / f"atm_{name}.npz"
    np.savez_compressed(out, **kept)
    return full_npz


def run_case(name: str, full_npz: Path, work: Path) -> None:
    case = CASES[name]
    lines = case_lines(case)
    text = workloads.format_gfall(lines)
    gf = work / f"{name}.gf"
    gf.write_text(text)
    dumps = work / f"dumps_{name}"
    dumps.mkdir(exist_ok=True)
    spec = work / f"{name}.spec"
    env = _env()
    env["SYNTHE_PY_STAGE_DUMPS"] = str(dumps)
    subprocess.run(
        [sys.executable, "-m", "synthe_py.cli", str(full_npz), str(gf),
         "--npz", str(full_npz), "--spec", str(spec),
         "--wl-start", repr(case["wl_start"]), "--wl-end", repr(case["wl_end"]),
         "--resolution", "300000", "--n-workers", "1",
         "--cache", str(work / "cache"), "--log-level", "WARNING",
         "--rhoxj", repr(float(case.get("rhoxj", 0.0))),
         "--microturb", repr(float(case.get("microturb", 0.0)))],
        check=True, env=env, cwd=work,
    )
    s3 = np.load(dumps / "stage_3_transp.npz")
    s4 = np.load(dumps / "stage_4_asynth.npz")
    s5 = np.load(dumps / "stage_5_rt.npz")
    spec_cols = np.loadtxt(spec)
    out = dict(
        gfall_sha256=np.array(hashlib.sha256(text.encode()).hexdigest()),
        wl_start=np.float64(case["wl_start"]), wl_end=np.float64(case["wl_end"]),
        resolution=np.float64(300000.0),
        rhoxj=np.float64(case.get("rhoxj", 0.0)), microturb=np.float64(case.get("microturb", 0.0)),
        wavelength=s5["wavelength"],
        line_indices=np.asarray(s3["line_indices"], dtype=np.int64),
        valid_mask=np.packbits(np.asarray(s3["valid_mask"], dtype=bool), axis=None),
        valid_shape=np.array(s3["valid_mask"].shape),
        flux_total_hz=s5["flux_total_hz"], flux_cont_hz=s5["flux_cont_hz"],
        spec=spec_cols,
    )
    transp = np.asarray(s3["transp"])
    asynth = np.asarray(s4["asynth"])
    if case.get("hydrogen") or case.get("helium"):
        # the line opacity the transfer sees: ASYNTH plus the hydrogen
        # profiles and the helium wings
        out["line_opacity"] = np.asarray(s5["line_opacity"])
    if name in LARGE_CASES:
        rng = np.random.default_rng(7)
        vi = np.argwhere(np.asarray(s3["valid_mask"]))
        pick = vi[rng.choice(vi.shape[0], size=min(4000, vi.shape[0]), replace=False)]
        out["transp_pairs"] = pick.astype(np.int64)
        out["transp_values"] = transp[pick[:, 0], pick[:, 1]]
        rows = np.array([0, 12, 24, 36, 48, 60, 71])
        out["asynth_rows"] = rows
        out["asynth"] = asynth[rows]
        out["cont_abs_rows"] = np.asarray(s5["cont_abs"])[rows]
        out["cont_scat_rows"] = np.asarray(s5["cont_scat"])[rows]
    else:
        out["transp"] = transp
        out["asynth"] = asynth
        out["cont_abs"] = np.asarray(s5["cont_abs"])
        out["cont_scat"] = np.asarray(s5["cont_scat"])
        out["stim"] = np.asarray(s4["stim"])
        out["bnu"] = np.asarray(s4["bnu"])
    np.savez_compressed(HERE / f"case_{name}.npz", **out)


def main(argv: list[str]) -> int:
    global REFERENCE
    if argv[:1] == ["--reference"]:
        REFERENCE = Path(argv[1])
        argv = argv[2:]
    wanted = argv or list(CASES)
    with tempfile.TemporaryDirectory(prefix="kgold_") as tmp:
        work = Path(tmp)
        built = {}
        for name in wanted:
            atm = CASES[name]["atm"]
            if atm not in built:
                built[atm] = build_atmosphere(atm, work)
            run_case(name, built[atm], work)
            print(f"wrote case_{name}.npz", flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main(sys.argv[1:]))
