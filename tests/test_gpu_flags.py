"""Internal-limit flags reach the caller on every path, also when no counters
are read (needs a GPU).

The planted fault is in the input, and the kernels' own check catches it: a
Doppler width of about 10 (v/c, a million times the physical one) gives
N10DOP = 10 * dop * R of about 3e7, beyond the 24-bit field of the pair
descriptor, so the pair setup raises FLAG_N10DOP_RANGE and drops the pair
before writing anything for it.  The populations are scaled by the same
factor, so XNFDOP = pop / (rho dop) and with it the TRANSP gates are as in
the physical case.  Nothing else in the path reads the Doppler width, so
every access stays in bounds.
"""

import dataclasses

import numpy as np
import pytest

from _cases import atm_path, golden, gfall_path, window
from kurucz_py_joss_submission_gb300 import _native
from kurucz_py_joss_submission_gb300.device import (DeviceAtmosphere, DeviceCatalog, DeviceGrid, Synthesizer,
                                                     check_flags, make_options)
from kurucz_py_joss_submission_gb300.io import atmosphere as atm_io
from kurucz_py_joss_submission_gb300.io.lines import atomic

pytestmark = pytest.mark.gpu

NAME = "tiny_500_501"


def _inputs(doppler_scale):
    w0, w1 = window(NAME)
    atm = atm_io.load_cached(atm_path(NAME))
    atm = dataclasses.replace(atm, doppler_per_ion=atm.doppler_per_ion * doppler_scale,
                              population_per_ion=atm.population_per_ion * doppler_scale)
    cat = atomic.load_catalog_window(gfall_path(NAME), w0, w1)
    return DeviceCatalog(cat), DeviceAtmosphere(atm), DeviceGrid(golden(NAME)["wavelength"])


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_flag_surfaces_without_stats(precision):
    check_flags()  # start from a clear sticky word
    dcat, datm, dgrid = _inputs(1e6)
    syn = Synthesizer(dcat, datm, dgrid, make_options(precision=precision), keep_asynth=False)
    syn.run()  # no stats: the call itself returns KS_OK, asynchronously
    with pytest.raises(_native.KsError) as e:
        check_flags()
    assert e.value.code == 7 and "N10DOP" in str(e.value)
    check_flags()  # taken and cleared by the check above
    # the same call with stats reports its own flags directly, and also
    # leaves them in the sticky word (every flag since the last check)
    with pytest.raises(_native.KsError):
        syn.run(stats=True)
    with pytest.raises(_native.KsError):
        check_flags()
    check_flags()


def test_graph_replay_keeps_flags():
    """A captured synthesis replayed without stats: the flag is still seen."""
    import torch

    check_flags()
    dcat, datm, dgrid = _inputs(1e6)
    syn = Synthesizer(dcat, datm, dgrid, make_options(), keep_asynth=False)
    syn.run()
    torch.cuda.synchronize()
    with pytest.raises(_native.KsError):
        check_flags()
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        syn.run()
    g.replay()
    with pytest.raises(_native.KsError):
        check_flags()


def test_clean_run_raises_nothing():
    check_flags()
    dcat, datm, dgrid = _inputs(1.0)
    syn = Synthesizer(dcat, datm, dgrid, make_options(), keep_asynth=False)
    for _ in range(3):
        syn.run()
    assert _native.check_device_flags(None) == 0
    assert np.all(np.isfinite(syn.flux_total.cpu().numpy()))
