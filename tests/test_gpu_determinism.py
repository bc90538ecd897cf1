"""Repeat runs give the same bits (needs a GPU).

Every sum in the accumulation has a fixed order except one: in the short-pair
loop the lanes of a warp add into the warp's own shared-memory copy of the
tile with shared-memory atomics, and two lanes can hit one bin in the same
step.  The hardware applies those in one order, but CUDA does not promise
which.  This test is the evidence that, on this GPU and build, the results
do not change from run to run: every golden case, both precisions, 20
repeats, ASYNTH and both fluxes compared bit for bit with the first run.
"""

import numpy as np
import pytest
import torch

from _cases import atm_path, available_cases, device_options, gfall_path, golden, window
from kurucz_py_joss_submission_gb300.device import (DeviceAtmosphere, DeviceCatalog, DeviceGrid, Synthesizer,
                                                     make_options)
from kurucz_py_joss_submission_gb300.io import atmosphere as atm_io
from kurucz_py_joss_submission_gb300.io.lines import atomic

pytestmark = pytest.mark.gpu

REPEATS = 20


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("name", available_cases())
def test_repeats_are_bit_identical(name, precision):
    w0, w1 = window(name)
    cat = atomic.load_catalog_window(gfall_path(name), w0, w1)
    atm = atm_io.load_cached(atm_path(name))
    syn = Synthesizer(DeviceCatalog(cat), DeviceAtmosphere(atm), DeviceGrid(golden(name)["wavelength"]),
                      make_options(precision=precision, **device_options(name)))
    syn.run()
    torch.cuda.synchronize()
    a0, f0, c0 = syn.asynth.clone(), syn.flux_total.clone(), syn.flux_cont.clone()
    for _ in range(REPEATS - 1):
        syn.asynth.fill_(-1.0)
        syn.run()
        torch.cuda.synchronize()
        assert torch.equal(syn.asynth, a0)
        assert torch.equal(syn.flux_total, f0)
        assert torch.equal(syn.flux_cont, c0)
    assert bool(torch.all(torch.isfinite(f0)))
