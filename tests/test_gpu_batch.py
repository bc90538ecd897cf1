"""Batched form against single syntheses (needs a GPU): every job of a batch
plan (one persistent launch per stage over all jobs), eager and replayed from
the captured graph, equals a standalone ks_synthesize of the same
atmosphere, window, lines and options bit for bit."""

import numpy as np
import pytest
import torch

from _cases import atm_path, gfall_path
from kurucz_py_joss_submission_gb300 import batch
from kurucz_py_joss_submission_gb300.device import (DeviceAtmosphere, DeviceCatalog, DeviceGrid,
                                                     Synthesizer, make_options)
from kurucz_py_joss_submission_gb300.io import atmosphere as atm_io
from kurucz_py_joss_submission_gb300.io.lines import atomic

pytestmark = pytest.mark.gpu

JOBS = [batch.Job(0, 500.5, 501.5), batch.Job(1, 502.0, 505.0), batch.Job(0, 506.0, 509.9),
        batch.Job(1, 500.2, 500.9), batch.Job(0, 503.3, 503.4)]


OPTION_SETS = [{}, dict(tile_bins=512, warps_per_tile=4, long_class=10), dict(transfer_path=1),
               dict(rhoxj=0.3, microturb_kms=2.0)]


def _inputs():
    cat = atomic.load_catalog(gfall_path("window_500_510"))
    srt = cat.take(np.argsort(cat.wavelength, kind="stable"))
    atms = [atm_io.load_cached(atm_path("tiny_500_501")), atm_io.load_cached(atm_path("strong_600_601"))]
    return srt, atms


def _single(srt, atms, j, precision, options):
    sub = atomic.filter_by_range(srt, j.wl_start, j.wl_end)
    g = batch.wavelength_grid(j.wl_start, j.wl_end)
    syn = Synthesizer(DeviceCatalog(sub), DeviceAtmosphere(atms[j.atmosphere]), DeviceGrid(g),
                      make_options(precision=precision, **options), keep_asynth=False)
    st = syn.run(stats=True)
    torch.cuda.synchronize()
    return syn, st


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("opt_i", range(len(OPTION_SETS)))
def test_batch_jobs_equal_single_syntheses(precision, opt_i):
    options = OPTION_SETS[opt_i]
    if precision == "fp64" and "transfer_path" in options:
        pytest.skip("transfer_path selects between the single-precision transfers")
    srt, atms = _inputs()
    bs = batch.BatchSynthesizer(DeviceCatalog(srt), atms, JOBS, precision=precision, options=options)
    bs.capture()
    for f in bs.flux_total + bs.flux_cont:
        f.zero_()
    bs.replay(check=True)
    torch.cuda.synchronize()
    evals = 0
    for i, j in enumerate(JOBS):
        syn, st = _single(srt, atms, j, precision, options)
        evals += st["evaluations"]
        assert torch.equal(bs.flux_total[i], syn.flux_total), i
        assert torch.equal(bs.flux_cont[i], syn.flux_cont), i
    st = bs.run(stats=True)
    assert st["evaluations"] == evals
    assert st["device_flags"] == 0


def test_job_groups_give_the_same_spectra():
    """Jobs split over three plans on streams of their own: same bits."""
    srt, atms = _inputs()
    dcat = DeviceCatalog(srt)
    one = batch.BatchSynthesizer(dcat, atms, JOBS)
    one.run()
    three = batch.BatchSynthesizer(dcat, atms, JOBS, groups=3)
    three.capture()
    three.replay(check=True)
    torch.cuda.synchronize()
    assert sorted(i for g in three.group_jobs for i in g) == list(range(len(JOBS)))
    for a, b in zip(one.flux_total + one.flux_cont, three.flux_total + three.flux_cont):
        assert torch.equal(a, b)
    assert three.run(stats=True)["evaluations"] == one.run(stats=True)["evaluations"]


def test_batch_through_the_c_entry_point():
    """ks_synthesize_batch (create, run, free in one call) gives the plan's result."""
    import ctypes as C

    from kurucz_py_joss_submission_gb300 import _native
    from kurucz_py_joss_submission_gb300.device import _ptr, stream_handle

    srt, atms = _inputs()
    dcat = DeviceCatalog(srt)
    bs = batch.BatchSynthesizer(dcat, atms, JOBS)
    bs.run()
    torch.cuda.synchronize()
    want = [f.clone() for f in bs.flux_total]
    for f in bs.flux_total:
        f.zero_()
    lib = _native.load()
    st = _native.KsStats()
    _native.check(lib.ks_synthesize_batch(C.byref(dcat.rec), bs.job_recs, len(JOBS), C.byref(bs.options),
                                          _ptr(bs.workspace), bs.workspace.numel(), C.byref(st),
                                          stream_handle()))
    torch.cuda.synchronize()
    for a, b in zip(want, bs.flux_total):
        assert torch.equal(a, b)
    assert st.kernel_launches == 15 and st.evaluations > 0


def test_batch_rejects_a_slice_outside_the_list():
    import ctypes as C

    from kurucz_py_joss_submission_gb300 import _native

    srt, atms = _inputs()
    dcat = DeviceCatalog(srt)
    bs = batch.BatchSynthesizer(dcat, atms, JOBS[:1])
    bad = (_native.KsJob * 1)()
    bad[0] = bs.job_recs[0]
    bad[0].line_count = dcat.n_lines + 1
    lib = _native.load()
    n = C.c_size_t()
    assert lib.ks_batch_workspace_size(C.byref(dcat.rec), bad, 1, C.byref(bs.options), C.byref(n)) == 1
    assert b"outside" in lib.ks_last_error()
