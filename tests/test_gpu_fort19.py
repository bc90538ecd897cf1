"""fort.19 NORMAL lines on the GPU (needs a GPU).

Metal lines with NBLO/NBUP set leave TRANSP/ASYNTH for fort.19 and get the
profiles of _add_fort19_asynth (engine/opacity.py:1335-1488), added to
ASYNTH before the hydrogen lines.  Checked against the reference's golden
(through the parity tests' fused FP64/mixed runs, which take every golden
case) and here against the oracle where no golden exists: microturbulence
in the lines' Doppler widths, damping large enough for the Voigt branch
(ADAMP >= 0.2), a line centred below the grid (the reference's clamped
KAPCEN bin and wing from bin 0), a raised cutoff, and autoionizing lines
(TYPE 1) interleaved with them, one of them below the grid (its centre value
on the last grid point, as the reference's Python index -1 puts it), and
merged-continuum records (LABELP CONTINUU), one of them below the grid.

Tolerance: FP64 cube within 1e-11 relative of the oracle's.
"""

import numpy as np
import pytest
import torch

from _cases import atm_path, available_cases
from kurucz_py_joss_submission_gb300 import workloads
from kurucz_py_joss_submission_gb300.device import (DeviceAtmosphere, DeviceCatalog, DeviceGrid,
                                                     Synthesizer, make_options)
from kurucz_py_joss_submission_gb300.engine.continuum import build_depth_continuum
from kurucz_py_joss_submission_gb300.io import atmosphere as atm_io
from kurucz_py_joss_submission_gb300.io.lines import atomic
from oracle import fort19, gfall, oracle

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-11
ATM = atm_path("tiny_500_501")


def gpu_cubes(cat, atm, grid, **opt):
    dcat = DeviceCatalog(cat)
    syn = Synthesizer(dcat, DeviceAtmosphere(atm), DeviceGrid(grid), make_options(precision="fp64", **opt))
    st = syn.run(stats=True)
    assert st["device_flags"] == 0
    with_f = syn.asynth.cpu().numpy()
    n = dcat.rec.n_f19
    dcat.rec.n_f19 = 0
    syn.run()
    torch.cuda.synchronize()
    without = syn.asynth.cpu().numpy()
    dcat.rec.n_f19 = n
    return dcat, with_f, without


def draw(w0, w1, seed, gw_shift=0.0, extra=None, aut=False):
    d = workloads.random_atomic_lines(80, w0 - 0.15, w1 + 0.15, seed=seed)
    lo, up = d.levels()
    lo, up = lo.copy(), up.copy()
    lo[::3], up[::3] = 4, 6
    d.n_lower, d.n_upper = lo, up
    idx = np.arange(0, len(d), 3)
    d.log_gf[idx] = np.maximum(d.log_gf[idx], -0.5)
    d.e_lower_cm[idx] = np.minimum(d.e_lower_cm[idx], 20000.0)
    d.log_gamma_vdw[idx] += gw_shift
    if aut:
        # autoionizing lines between them (interleaved in fort.19 order)
        ia = np.arange(1, len(d), 4)
        tag = np.array([""] * len(d), dtype=object)
        tag[ia] = "AUT"
        d.tag = tag
        d.log_gamma_rad[ia] = 11.0
        d.log_gamma_stark[ia] = np.where(np.arange(ia.size) % 2 == 0, -0.5, 0.3)
        d.log_gamma_vdw[ia] = 0.3
        d.log_gf[ia] = np.minimum(d.log_gf[ia], -1.0) - 12.0
    if extra is not None:
        d = workloads.merge_lines(d, extra)
    return d


def continuum_records(w0):
    """Merged-continuum records (LABELP CONTINUU, NLAST = XJP): one below
    the grid, two inside it."""
    wl = np.array([w0 - 0.08, w0 + 0.12, w0 + 0.45])
    z = np.zeros(3)
    return workloads.LineDraw(wavelength_nm=wl, log_gf=np.array([-16.0, -15.5, -16.5]),
                              code=np.full(3, 26.00), e_lower_cm=np.full(3, 1500.0),
                              log_gamma_rad=z + 8.0, log_gamma_stark=z - 5.0, log_gamma_vdw=z - 7.5,
                              labelp=np.array(["CONTINUU"] * 3, dtype=object), xjp=np.array([40.0, 50.0, 30.0]))


def below_grid_aut(w0):
    """One autoionizing Fe I line below the grid: the reference puts its centre
    value on the last grid point (Python index -1)."""
    d = below_grid_line(w0)
    d.n_lower = d.n_upper = None
    d.tag = np.array(["AUT"], dtype=object)
    d.log_gamma_rad[:] = 11.0
    d.log_gamma_stark[:] = -0.5
    d.log_gamma_vdw[:] = 0.3
    d.log_gf[:] = -13.0
    return d


def below_grid_line(w0):
    """One strong NB-tagged Fe I line 0.02 nm below the grid start."""
    d = workloads.random_atomic_lines(1, w0 - 0.03, w0 - 0.02, seed=5)
    d.log_gf[:] = 0.5
    d.e_lower_cm[:] = 1000.0
    d.code[:] = 26.00
    d.n_lower, d.n_upper = np.array([2], np.int32), np.array([7], np.int32)
    return d


CASES = {
    "micro": (500.0, 500.8, dict(seed=31), {"microturb_kms": 2.0}),
    "voigt_branch": (500.0, 500.8, dict(seed=32, gw_shift=3.0), {}),
    "below_grid": (500.0, 500.8, dict(seed=33, extra="below"), {}),
    "cutoff": (500.0, 500.8, dict(seed=34), {"cutoff": 1e-2}),
    # NORMAL and autoionizing lines interleaved; an autoionizing line below the grid
    "with_aut": (500.0, 500.8, dict(seed=35, aut=True), {}),
    "aut_below": (500.0, 500.8, dict(seed=36, aut=True, extra="below_aut"), {}),
    # merged-continuum ramps with NORMAL and autoionizing lines
    "continuum": (505.5, 506.6, dict(seed=37, aut=True, extra="continuum"), {}),
}


@pytest.mark.parametrize("key", sorted(CASES))
def test_fp64_matches_oracle(key, tmp_path):
    w0, w1, kw, opt = CASES[key]
    kw = dict(kw)
    extra = kw.pop("extra", None)
    if extra == "below":
        kw["extra"] = below_grid_line(w0)
    elif extra == "below_aut":
        kw["extra"] = below_grid_aut(w0)
    elif extra == "continuum":
        kw["extra"] = continuum_records(w0)
    p = tmp_path / "lines.gf"
    p.write_text(workloads.format_gfall(draw(w0, w1, **kw)))
    cat = atomic.load_catalog_window(p, w0, w1)
    grid = oracle.wavelength_grid(w0, w1, 300000.0)
    atm = atm_io.load_cached(ATM)
    dcat, with_f, without = gpu_cubes(cat, atm, grid, **opt)
    assert dcat.n_f19 > 10
    ocat = gfall.filter_window(gfall.parse_gfall(p, oracle.tables()["potion"]), w0, w1)
    assert np.array_equal(ocat["wavelength"], cat.wavelength)
    ca, cs = build_depth_continuum(atm, grid, precision="fp64")
    term = fort19.asynth_term(dict(ocat, center=oracle.center_indices(grid, ocat["wavelength"])),
                              oracle.load_atmosphere(ATM), grid, ca + cs, cutoff=opt.get("cutoff", 1e-3),
                              microturb_kms=opt.get("microturb_kms", 0.0))
    assert np.count_nonzero(term) > 1000
    ref = without + term
    assert float(np.max(np.abs(with_f - ref) / np.maximum(np.abs(ref), 1e-300))) < FP64_TOL
    c = oracle.center_indices(grid, ocat["wavelength"])
    if key == "below_grid":
        assert np.any(c[fort19.normal_rows(dict(ocat, center=c))] < 0)
    if key.startswith("aut") or key == "with_aut":
        assert fort19.aut_rows(ocat).size >= 10
    if key == "aut_below":
        assert np.any(c[fort19.aut_rows(ocat)] < 0)
    if key == "continuum":
        assert fort19.cont_rows(ocat).size == 3 and dcat.t["f19_kind"].eq(2).sum().item() == 3


def test_more_lines_than_workspace_scratch(tmp_path):
    """300 fort.19 lines (beyond the 256 a workspace holds scratch for): the
    synthesis allocates the rest on its stream and matches the oracle."""
    w0, w1 = 500.0, 500.6
    d = workloads.random_atomic_lines(360, w0 - 0.15, w1 + 0.15, seed=38)
    d.n_lower, d.n_upper = np.full(len(d), 3, np.int32), np.full(len(d), 5, np.int32)
    p = tmp_path / "lines.gf"
    p.write_text(workloads.format_gfall(d))
    cat = atomic.load_catalog_window(p, w0, w1)
    grid = oracle.wavelength_grid(w0, w1, 300000.0)
    atm = atm_io.load_cached(ATM)
    dcat, with_f, without = gpu_cubes(cat, atm, grid)
    assert dcat.n_f19 > 256
    ocat = gfall.filter_window(gfall.parse_gfall(p, oracle.tables()["potion"]), w0, w1)
    ca, cs = build_depth_continuum(atm, grid, precision="fp64")
    term = fort19.asynth_term(dict(ocat, center=oracle.center_indices(grid, ocat["wavelength"])),
                              oracle.load_atmosphere(ATM), grid, ca + cs)
    ref = without + term
    assert float(np.max(np.abs(with_f - ref) / np.maximum(np.abs(ref), 1e-300))) < FP64_TOL
