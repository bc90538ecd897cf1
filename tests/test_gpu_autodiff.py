"""Adjoint gradients of the differentiable form against central finite
differences of the same (FP64, exactly solved) synthesis (needs a GPU)."""

import numpy as np
import pytest
import torch

from _cases import atm_path, gfall_path, golden, window
from kurucz_py_joss_submission_gb300 import autodiff
from kurucz_py_joss_submission_gb300.io import atmosphere as atm_io
from kurucz_py_joss_submission_gb300.io.lines import atomic

pytestmark = pytest.mark.gpu


def _setup(name):
    w0, w1 = window(name)
    cat = atomic.load_catalog_window(gfall_path(name), w0, w1, sort=True)
    atm = atm_io.load_cached(atm_path(name))
    return autodiff.DiffSynthesizer(cat, atm, golden(name)["wavelength"]), len(cat)


def _loss(ft, fc, target):
    return torch.sum((ft / fc - target) ** 2)


@pytest.mark.parametrize("name", ["tiny_500_501", "uv_300_302"])
def test_adjoint_matches_finite_differences(name):
    ds, n = _setup(name)
    dev = ds.flux_total.device
    zeros = [torch.zeros(n, dtype=torch.float64, device=dev, requires_grad=True) for _ in range(4)]
    ft0, fc0 = ds.forward()
    target = (ft0 / fc0).detach() * 0.98 + 0.01
    ft, fc = autodiff.synthesize(ds, *zeros)
    loss = _loss(ft, fc, target)
    loss.backward()
    grads = [z.grad.cpu().numpy() for z in zeros]
    assert all(np.all(np.isfinite(g)) for g in grads)
    rng = np.random.default_rng(7)
    h = 1e-3
    checked = 0
    errs = []
    for p in range(4):
        g = grads[p]
        # the most sensitive lines of this parameter, plus random ones
        cand = list(np.argsort(-np.abs(g))[:6]) + list(rng.integers(0, n, 4))
        for i in cand:
            vals = []
            for s in (+1, -1):
                d = [torch.zeros(n, dtype=torch.float64, device=dev) for _ in range(4)]
                d[p][i] = s * h
                a, b = ds.forward(*d)
                vals.append(_loss(a, b, target).item())
            fd = (vals[0] - vals[1]) / (2 * h)
            scale = max(abs(fd), abs(g[i]), 1e-12 * abs(loss.item()) + 1e-300)
            errs.append(abs(fd - g[i]) / scale)
            checked += 1
    errs = np.array(errs)
    # gates and wing reach are steps the adjoint holds fixed: most parameters
    # agree closely, a few may differ where a step is crossed within +-h
    assert np.median(errs) < 1e-2, errs
    assert np.mean(errs < 5e-2) >= 0.8, errs


def test_adjoint_matches_differenced_oracle():
    """The adjoint against central differences of the oracle -- the C
    restatement of the reference path, run independently of this library --
    with the JOSH system solved exactly (oracle.set_exact_sweeps; the
    reference's FP32 sweep with its 1e-5 stop is not smooth enough to
    difference).  h = 1e-4 dex on the most sensitive lines of each parameter
    class (log gf and the three log damping constants) and on random ones.
    The TRANSP gates and the integer wing reach are steps that the adjoint
    holds fixed; the oracle reports every pair's validity and reach, so a
    parameter whose +-h runs differ there has crossed a step and is left out
    (the strongest lines, with the longest far wings, often do).  Every other
    parameter must agree to 1e-4 relative (median below 1e-6)."""
    from oracle import gfall, oracle

    name = "tiny_500_501"
    ds, n = _setup(name)
    dev = ds.flux_total.device
    zeros = [torch.zeros(n, dtype=torch.float64, device=dev, requires_grad=True) for _ in range(4)]
    ft0, fc0 = ds.forward()
    target = ((ft0 / fc0).detach() * 0.98 + 0.01).cpu().numpy()
    ft, fc = autodiff.synthesize(ds, *zeros)
    loss = torch.sum((ft / fc - torch.as_tensor(target, device=dev)) ** 2)
    loss.backward()
    grads = [z.grad.cpu().numpy() for z in zeros]

    # the oracle's catalog in the GPU's (stable, wavelength-sorted) order
    w0, w1 = window(name)
    tb = oracle.tables()
    ocat = gfall.filter_window(gfall.parse_gfall(gfall_path(name), tb["potion"]), w0, w1)
    order = np.argsort(ocat["wavelength"], kind="stable")
    ocat = {k: v[order] for k, v in ocat.items()}
    assert np.array_equal(ocat["wavelength"], ds.cat.host.wavelength)
    atm = oracle.load_atmosphere(atm_path(name))
    cols = ("log_gf", "gamma_rad", "gamma_stark", "gamma_vdw")

    def oracle_run(p, i, dex):
        c = {k: v.copy() for k, v in ocat.items()}
        if p == 0:
            c["log_gf"][i] += dex
        else:
            c[cols[p]][i] *= 10.0 ** dex
        r = oracle.synthesize(atm, c, w0, w1, tb=tb)
        return (float(np.sum((r["flux_total_hz"] / r["flux_cont_hz"] - target) ** 2)),
                r["reach"][i].copy(), r["valid_mask"][i].copy())

    h = 1e-4
    rng = np.random.default_rng(11)
    errs, stepped = [], 0
    oracle.set_exact_sweeps(True)
    try:
        for p in range(4):
            g = grads[p]
            for i in list(np.argsort(-np.abs(g))[:6]) + list(rng.integers(0, n, 8)):
                lp, reach_p, valid_p = oracle_run(p, i, h)
                lm, reach_m, valid_m = oracle_run(p, i, -h)
                if not (np.array_equal(reach_p, reach_m) and np.array_equal(valid_p, valid_m)):
                    stepped += 1
                    continue
                fd = (lp - lm) / (2 * h)
                scale = max(abs(fd), abs(g[i]))
                if scale * h <= 1e-11 * float(loss.item()):
                    continue  # below what the difference resolves
                errs.append(abs(fd - g[i]) / scale)
    finally:
        oracle.set_exact_sweeps(False)
    errs = np.array(errs)
    assert errs.size >= 12, (errs, stepped)
    assert np.median(errs) < 1e-6, errs
    assert np.all(errs < 1e-4), errs
