"""Batched form against single syntheses (needs a GPU): every job of a batch,
eager and replayed from the captured graph, equals a standalone
ks_synthesize of the same atmosphere, window and lines bit for bit."""

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


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_batch_jobs_equal_single_syntheses(precision):
    cat = atomic.load_catalog(gfall_path("window_500_510"))
    srt = cat.take(np.argsort(cat.wavelength, kind="stable"))
    atms = [atm_io.load_cached(atm_path("tiny_500_501")), atm_io.load_cached(atm_path("strong_600_601"))]
    dcat = DeviceCatalog(srt)
    bs = batch.BatchSynthesizer(dcat, atms, JOBS, precision=precision, n_streams=3)
    bs.capture()
    for f in bs.flux_total + bs.flux_cont:
        f.zero_()
    bs.replay()
    torch.cuda.synchronize()
    for i, j in enumerate(JOBS):
        sub = atomic.filter_by_range(srt, j.wl_start, j.wl_end)
        g = batch.wavelength_grid(j.wl_start, j.wl_end)
        syn = Synthesizer(DeviceCatalog(sub), DeviceAtmosphere(atms[j.atmosphere]), DeviceGrid(g),
                          make_options(precision=precision), keep_asynth=False)
        syn.run()
        torch.cuda.synchronize()
        assert torch.equal(bs.flux_total[i], syn.flux_total), i
        assert torch.equal(bs.flux_cont[i], syn.flux_cont), i
