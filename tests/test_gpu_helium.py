"""Helium lines on the GPU (needs a GPU).

The fused synthesis adds the reference's helium wing pass (line types
-3/-4/-6; engine/opacity.py:2515-3590, Voigt wings of :996-1061) to the line
opacity as AHE x STIM (:3650-3660).  Checked against
* the reference's goldens (He I 447.1 nm, He II 468.6 nm in a 20,000 K
  atmosphere): FP64 cube and fluxes, mixed path within the flux contract;
* the oracle (bit-exact with those goldens) where no golden exists: two
  helium lines with overlapping wings (catalog-order sums), a 3He line
  (kappa / 1.155, Doppler width x 1.155), a raised cutoff, and a line whose
  centre lies outside the grid (the reference skips it).

Tolerances: FP64 cube within 1e-11 relative of the reference / oracle,
fluxes within 1e-9 of the continuum; mixed F/Fc within 1e-4.
"""

import dataclasses

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
from oracle import gfall, helium, oracle

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-11
FLUX_TOL = 1e-9
NORM_TOL = 1e-4
HELIUM_CASES = [c for c in ("hei_447", "heii_468") if c in available_cases()]
ATM = atm_path("hei_447")


def gpu_cubes(cat, atm, grid, precision="fp64", **opt):
    """Line opacity cube and fluxes with and without the helium lines."""
    dcat = DeviceCatalog(cat)
    syn = Synthesizer(dcat, DeviceAtmosphere(atm), DeviceGrid(grid), make_options(precision=precision, **opt))
    st = syn.run(stats=True)
    assert st["device_flags"] == 0
    with_he = syn.asynth.cpu().numpy().astype(np.float64)
    flux = (syn.flux_total.cpu().numpy(), syn.flux_cont.cpu().numpy())
    n = dcat.rec.n_helium
    dcat.rec.n_helium = 0
    syn.run()
    torch.cuda.synchronize()
    without = syn.asynth.cpu().numpy().astype(np.float64)
    dcat.rec.n_helium = n
    return dcat, with_he, without, flux


def rel(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


@pytest.mark.parametrize("name", HELIUM_CASES)
def test_fp64_matches_reference_goldens(name):
    g = golden(name)
    w0, w1 = window(name)
    cat = atomic.load_catalog_window(gfall_path(name), w0, w1)
    dcat, with_he, without, (ft, fc) = gpu_cubes(cat, atm_io.load_cached(atm_path(name)), g["wavelength"])
    assert dcat.n_helium == 1
    assert rel(with_he, g["line_opacity"]) < FP64_TOL
    assert rel(without, g["asynth"]) < 1e-12
    assert not np.array_equal(with_he, without)
    assert float(np.max(np.abs(ft - g["flux_total_hz"]) / g["flux_cont_hz"])) < FLUX_TOL


@pytest.mark.parametrize("name", HELIUM_CASES)
def test_mixed_within_contract(name):
    g = golden(name)
    w0, w1 = window(name)
    cat = atomic.load_catalog_window(gfall_path(name), w0, w1)
    _, with_he, without, (ft, fc) = gpu_cubes(cat, atm_io.load_cached(atm_path(name)), g["wavelength"],
                                              precision="mixed")
    nf_ref = g["flux_total_hz"] / g["flux_cont_hz"]
    assert float(np.max(np.abs(ft / fc - nf_ref) / np.maximum(np.abs(nf_ref), 1e-3))) <= NORM_TOL
    assert not np.array_equal(with_he, without)


def oracle_cube(cat_path, w0, w1, grid, cutoff=1e-3, types=None):
    ocat = gfall.filter_window(gfall.parse_gfall(cat_path, oracle.tables()["potion"]), w0, w1)
    lt = ocat["line_type"].copy()
    if types:
        for row, t in types.items():
            lt[row] = t
    c = dict(wavelength=ocat["wavelength"], gf=10.0 ** ocat["log_gf"], elo=ocat["excitation_energy"],
             gamma_rad=ocat["gamma_rad"], gamma_stark=ocat["gamma_stark"], gamma_vdw=ocat["gamma_vdw"],
             ion_stage=ocat["ion_stage"], line_type=lt, center=oracle.center_indices(grid, ocat["wavelength"]))
    atm = oracle.load_atmosphere(ATM)
    ca, cs = build_depth_continuum(atm_io.load_cached(ATM), grid, precision="fp64")
    return helium.line_opacity(c, atm, grid, ca + cs, cutoff=cutoff), ocat


def he_pair(shift=0.04, dlog=-0.6):
    """He I 447.27 nm and a copy of it `shift` nm redder, `dlog` dex weaker."""
    d = workloads.helium_lines(447.0, 447.5)
    e = dataclasses.replace(d, wavelength_nm=d.wavelength_nm + shift, log_gf=d.log_gf + dlog)
    return workloads.merge_lines(d, e)


CASES = {
    # two helium lines whose wings overlap: per-point sums in catalog order
    "pair": (447.0, 447.6, he_pair, {}, None),
    # the same pair with a raised cutoff (shorter walks, gates closer)
    "pair_cutoff": (447.0, 447.6, he_pair, {"cutoff": 1e-2}, None),
    # 3He: the first helium line retyped -4 on both sides
    "he3": (447.0, 447.6, he_pair, {}, "first"),
    # centre outside the grid: the reference skips the line
    "off_grid": (447.35, 447.9, lambda: workloads.helium_lines(447.0, 447.5), {}, None),
}


@pytest.mark.parametrize("key", sorted(CASES))
def test_fp64_matches_oracle(key, tmp_path):
    w0, w1, make, opt, retype = CASES[key]
    metals = workloads.random_atomic_lines(60, w0 - 0.15, w1 + 0.15, seed=23)
    p = tmp_path / "lines.gf"
    p.write_text(workloads.format_gfall(workloads.merge_lines(metals, make())))
    cat = atomic.load_catalog_window(p, w0, w1)
    grid = oracle.wavelength_grid(w0, w1, 300000.0)
    types = None
    if retype:
        row = int(np.flatnonzero(np.isin(cat.line_types, (-3, -4, -6)))[0])
        cat = dataclasses.replace(cat, line_types=np.where(np.arange(len(cat)) == row, -4, cat.line_types)
                                  .astype(cat.line_types.dtype))
        types = {row: -4}
    ref, ocat = oracle_cube(p, w0, w1, grid, cutoff=opt.get("cutoff", 1e-3), types=types)
    assert np.array_equal(ocat["wavelength"], cat.wavelength)   # same rows on both sides
    dcat, with_he, without, _ = gpu_cubes(cat, atm_io.load_cached(ATM), grid, **opt)
    if key == "off_grid":
        assert dcat.n_helium == 1 and np.count_nonzero(ref) == 0
        assert np.array_equal(with_he, without)
        return
    assert np.count_nonzero(ref) > 100
    assert rel(with_he, without + ref) < FP64_TOL
