"""Hydrogen line opacity on the GPU (needs a GPU).

The fused synthesis adds the HPROF4 profiles of the catalog's hydrogen lines
to the line opacity cube before the transfer (engine/opacity.py:1706-1884,
:2465-2503).  Checked against
* the reference's Balmer goldens (H beta, H gamma windows): FP64 cube and
  fluxes, mixed path within the flux contract;
* the oracle (bit-exact with those goldens) on windows the goldens do not
  cover: H alpha (fine-structure components), Lyman alpha and beta (the
  Lyman cutoff tables and the quasi-static cut), the high Balmer members
  (series-neighbour cuts, the merge taper), a line centred outside the grid,
  microturbulence and a raised cutoff.

Tolerances: FP64 cube within 1e-11 relative of the oracle's (CUDA's pow, exp
and log against numpy's in the profile), fluxes within 1e-9 of the continuum;
the mixed path within the flux contract of the parity tests (1e-4 on F/Fc).
"""

import numpy as np
import pytest
import torch

from _cases import atm_path, available_cases, gfall_path, golden, window
from kurucz_py_joss_submission_gb300 import workloads
from kurucz_py_joss_submission_gb300.device import (DeviceAtmosphere, DeviceCatalog, DeviceGrid,
                                                     Synthesizer, make_options)
from kurucz_py_joss_submission_gb300.engine.continuum import build_depth_continuum
from kurucz_py_joss_submission_gb300.io import atmosphere as atm_io
from kurucz_py_joss_submission_gb300.io.lines import atomic
from oracle import gfall, hydrogen, oracle

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-11
FLUX_TOL = 1e-9
NORM_TOL = 1e-4
ATM = atm_path("hbeta_486") if "hbeta_486" in available_cases() else None
HYDROGEN_CASES = [c for c in ("hbeta_486", "hgamma_434") if c in available_cases()]

_EHYD = workloads._EHYD


def lyman_lines(upper):
    """Lyman lines 1 -> m as gfall records (NBLO = 1, NBUP = m)."""
    log_gf = {2: -0.080, 3: -0.802, 4: -1.184}
    m = np.asarray(sorted(upper), dtype=np.int32)
    e_lo = np.zeros(m.size)
    wl = 1.0e7 / (np.array([_EHYD[k - 1] for k in m]) - e_lo)
    z = np.zeros(m.size)
    return workloads.LineDraw(wavelength_nm=wl, log_gf=np.array([log_gf[k] for k in m]),
                              code=np.full(m.size, 1.00), e_lower_cm=e_lo, log_gamma_rad=z + 8.79,
                              log_gamma_stark=z - 4.5, log_gamma_vdw=z - 7.5,
                              n_lower=np.full(m.size, 1, np.int32), n_upper=m)


def write_catalog(tmp_path, draw, w0, w1):
    p = tmp_path / "lines.gf"
    p.write_text(workloads.format_gfall(draw))
    cat = atomic.load_catalog_window(p, w0, w1)
    ocat = gfall.filter_window(gfall.parse_gfall(p, oracle.tables()["potion"]), w0, w1)
    return cat, ocat


def gpu_cubes(cat, atm, grid, precision="fp64", **opt):
    """Line opacity cube and fluxes with and without the hydrogen lines."""
    dcat = DeviceCatalog(cat)
    assert dcat.n_hydrogen > 0
    syn = Synthesizer(dcat, DeviceAtmosphere(atm), DeviceGrid(grid), make_options(precision=precision, **opt))
    st = syn.run(stats=True)
    assert st["device_flags"] == 0
    with_h = syn.asynth.cpu().numpy().astype(np.float64)
    flux = (syn.flux_total.cpu().numpy(), syn.flux_cont.cpu().numpy())
    dcat.rec.n_hydrogen = 0
    syn.run()
    torch.cuda.synchronize()
    without = syn.asynth.cpu().numpy().astype(np.float64)
    dcat.rec.n_hydrogen = dcat.n_hydrogen
    return with_h, without, flux


def oracle_ahline(ocat, grid, cont, microturb_kms=0.0, cutoff=1e-3):
    c = dict(wavelength=ocat["wavelength"], gf=10.0 ** ocat["log_gf"], elo=ocat["excitation_energy"],
             n_lower=ocat["n_lower"], n_upper=ocat["n_upper"], line_type=ocat["line_type"],
             ion_stage=ocat["ion_stage"], center=oracle.center_indices(grid, ocat["wavelength"]))
    return hydrogen.line_opacity(c, oracle.load_atmosphere(ATM), grid, cont, cutoff=cutoff,
                                 microturb_kms=microturb_kms)


def rel(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


@pytest.mark.parametrize("name", HYDROGEN_CASES)
def test_fp64_matches_reference_goldens(name):
    g = golden(name)
    w0, w1 = window(name)
    cat = atomic.load_catalog_window(gfall_path(name), w0, w1)
    atm = atm_io.load_cached(atm_path(name))
    with_h, without, (ft, fc) = gpu_cubes(cat, atm, g["wavelength"])
    assert rel(with_h, g["line_opacity"]) < FP64_TOL
    assert rel(without, g["asynth"]) < 1e-12
    assert not np.array_equal(with_h, without)
    assert float(np.max(np.abs(ft - g["flux_total_hz"]) / g["flux_cont_hz"])) < FLUX_TOL


@pytest.mark.parametrize("name", HYDROGEN_CASES)
def test_mixed_within_contract(name):
    g = golden(name)
    w0, w1 = window(name)
    cat = atomic.load_catalog_window(gfall_path(name), w0, w1)
    atm = atm_io.load_cached(atm_path(name))
    with_h, without, (ft, fc) = gpu_cubes(cat, atm, g["wavelength"], precision="mixed")
    nf_ref = g["flux_total_hz"] / g["flux_cont_hz"]
    assert float(np.max(np.abs(ft / fc - nf_ref) / np.maximum(np.abs(nf_ref), 1e-3))) <= NORM_TOL
    assert float(np.max(np.abs(ft / fc - nf_ref))) <= NORM_TOL
    assert not np.array_equal(with_h, without)


# windows without goldens, against the oracle
WINDOWS = {
    # H alpha: fine-structure components of an n -> n+1 line
    "halpha": (656.0, 657.2, lambda: workloads.balmer_lines([3]), {}),
    # H beta centred below the grid: only its red wing reaches it
    "hbeta_off_grid": (486.6, 487.3, lambda: workloads.balmer_lines([4, 5]), {}),
    # high Balmer members: series-neighbour cuts and the merge taper
    "balmer_high": (388.4, 390.2, lambda: workloads.balmer_lines([6, 7, 8]), {}),
    # Lyman alpha (Lyman cutoff tables, quasi-static cut) and beta
    "lyman_alpha": (121.2, 122.0, lambda: lyman_lines([2, 3]), {}),
    "lyman_beta": (102.3, 102.9, lambda: lyman_lines([2, 3, 4]), {}),
    # microturbulence and a raised cutoff
    "hbeta_micro": (485.9, 486.6, lambda: workloads.balmer_lines([4]), {"microturb_kms": 2.0, "cutoff": 3e-3}),
}


@pytest.mark.parametrize("key", sorted(WINDOWS))
def test_fp64_matches_oracle(key, tmp_path):
    w0, w1, make, opt = WINDOWS[key]
    metals = workloads.random_atomic_lines(60, w0, w1, seed=11)
    cat, ocat = write_catalog(tmp_path, workloads.merge_lines(metals, make()), w0, w1)
    atm = atm_io.load_cached(ATM)
    grid = oracle.wavelength_grid(w0, w1, 300000.0)
    with_h, without, _ = gpu_cubes(cat, atm, grid, **opt)
    ca, cs = build_depth_continuum(atm, grid, precision="fp64")
    ah = oracle_ahline(ocat, grid, ca + cs, microturb_kms=opt.get("microturb_kms", 0.0),
                       cutoff=opt.get("cutoff", 1e-3))
    assert np.count_nonzero(ah) > 100
    ref = without + ah
    assert rel(with_h, ref) < FP64_TOL
