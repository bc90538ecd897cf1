"""Depth-sharded synthesis against the unsharded one (needs a GPU).

All ranks run in one process on the one GPU (sharding.emulate): the same
ks_opacity / ks_transfer_opacity calls and exchange packing as a multi-GPU
run.  The stitched spectrum must be bit-identical to ks_synthesize."""

import numpy as np
import pytest
import torch

from _cases import atm_path, available_cases, device_options, golden, gfall_path, window
from kurucz_py_joss_submission_gb300 import sharding
from kurucz_py_joss_submission_gb300.device import (DeviceAtmosphere, DeviceCatalog, DeviceGrid,
                                                     Synthesizer, make_options)
from kurucz_py_joss_submission_gb300.io import atmosphere as atm_io
from kurucz_py_joss_submission_gb300.io.lines import atomic

pytestmark = pytest.mark.gpu


def _catalog(name):
    w0, w1 = window(name)
    return atomic.load_catalog_window(gfall_path(name), w0, w1)


@pytest.mark.parametrize("name", [c for c in available_cases() if c != "tiny_500_501"])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("world", [2, 3])
def test_sharded_spectrum_is_bit_identical(name, precision, world):
    g = golden(name)
    atm = atm_io.load_cached(atm_path(name))
    dc = DeviceCatalog(_catalog(name))
    opt = make_options(precision=precision, **device_options(name))
    syn = Synthesizer(dc, DeviceAtmosphere(atm), DeviceGrid(g["wavelength"]), opt, keep_asynth=False)
    st = syn.run(stats=True)
    torch.cuda.synchronize()
    ft, fc, evals = sharding.emulate(dc, atm, g["wavelength"], None, world,
                                     make_options(precision=precision, **device_options(name)))
    torch.cuda.synchronize()
    assert evals == st["evaluations"]
    assert torch.equal(ft, syn.flux_total)
    assert torch.equal(fc, syn.flux_cont)


def test_world_size_bounds():
    atm = atm_io.load_cached(atm_path("tiny_500_501"))
    g = golden("tiny_500_501")
    dc = DeviceCatalog(_catalog("tiny_500_501"))
    with pytest.raises(ValueError):
        sharding.ShardRank(dc, atm, g["wavelength"], None, 0, atm.layers + 1)
