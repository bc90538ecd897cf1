"""The no-allocation synthesis entry point against the workspace one.

ks_synthesize_noalloc serves callers that cannot allocate device memory
(a plug-in inside a host that owns all device memory, or a runtime reached
through an FFI with no CUDA allocator): it runs the same fused synthesis as
ks_synthesize, but in a fixed 64 MiB scratch array inside the library.  This
test calls it twice in a row through the C ABI and compares both results
with ks_synthesize on the same inputs; the kernels are deterministic, so the
fluxes must agree to 1e-12 (relative).  It also checks that the call takes
no device memory -- the device's free memory, and the used and reserved bytes
of the stream-ordered pool that cudaMallocAsync draws from, are the same
before and after it -- and that sizes beyond the scratch are rejected.  This
file is collected last so that a run stopping at the first failure has
already run every other test.
"""

import ctypes as C

import numpy as np
import pytest
import torch

from _cases import atm_path, gfall_path, golden, window
from kurucz_py_joss_submission_gb300 import _native
from kurucz_py_joss_submission_gb300.device import (DeviceAtmosphere, DeviceCatalog, DeviceGrid,
                                                     Synthesizer, make_options, stream_handle)
from kurucz_py_joss_submission_gb300.io import atmosphere as atm_io
from kurucz_py_joss_submission_gb300.io.lines import atomic

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _inputs(name):
    g = golden(name)
    w0, w1 = window(name)
    cat = atomic.load_catalog_window(gfall_path(name), w0, w1)
    atm = atm_io.load_cached(atm_path(name))
    return g, DeviceCatalog(cat), DeviceAtmosphere(atm), DeviceGrid(g["wavelength"])


def _noalloc(lib, dcat, datm, dgrid, opt):
    n = dgrid.n
    ft = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    fc = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    st = lib.ks_synthesize_noalloc(C.byref(dcat.rec), C.byref(datm.rec), C.byref(dgrid.rec), C.byref(opt),
                                   C.c_void_p(ft.data_ptr()), C.c_void_p(fc.data_ptr()), None,
                                   stream_handle())
    _native.check(st)
    torch.cuda.synchronize()
    return ft.cpu().numpy(), fc.cpu().numpy()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_noalloc_matches_workspace_entry_point_twice(precision):
    lib = _native.load()
    g, dcat, datm, dgrid = _inputs("uv_300_302")
    opt = make_options(precision=precision)
    ref = Synthesizer(dcat, datm, dgrid, opt, keep_asynth=False)
    ref.run()
    torch.cuda.synchronize()
    ft_ref = ref.flux_total.cpu().numpy()
    fc_ref = ref.flux_cont.cpu().numpy()
    for _ in range(2):
        ft, fc = _noalloc(lib, dcat, datm, dgrid, opt)
        assert np.all(np.isfinite(ft)) and np.all(np.isfinite(fc))
        assert float(np.max(np.abs(ft - ft_ref) / fc_ref)) <= TOL
        assert float(np.max(np.abs(fc / fc_ref - 1.0))) <= TOL


def _pool_bytes():
    """(reserved, used) bytes of the current device's default stream-ordered
    memory pool, read through the driver API (CU_MEMPOOL_ATTR_RESERVED_MEM_CURRENT
    = 5, CU_MEMPOOL_ATTR_USED_MEM_CURRENT = 7 in cuda.h)."""
    cu = C.CDLL("libcuda.so.1")
    dev = C.c_int()
    assert cu.cuCtxGetDevice(C.byref(dev)) == 0
    pool = C.c_void_p()
    assert cu.cuDeviceGetDefaultMemPool(C.byref(pool), dev) == 0
    out = []
    for attr in (5, 7):
        v = C.c_uint64()
        assert cu.cuMemPoolGetAttribute(pool, C.c_int(attr), C.byref(v)) == 0
        out.append(int(v.value))
    return tuple(out)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_noalloc_takes_no_device_memory(precision):
    lib = _native.load()
    _, dcat, datm, dgrid = _inputs("uv_300_302")
    opt = make_options(precision=precision)
    n = dgrid.n
    ft = torch.empty(n, dtype=torch.float64, device="cuda")
    fc = torch.empty(n, dtype=torch.float64, device="cuda")
    args = (C.byref(dcat.rec), C.byref(datm.rec), C.byref(dgrid.rec), C.byref(opt),
            C.c_void_p(ft.data_ptr()), C.c_void_p(fc.data_ptr()), None, stream_handle())
    # warm-up: the one-time set-up (tables, scratch address) and the lazy
    # loading of the kernels happen here
    _native.check(lib.ks_synthesize_noalloc(*args))
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    pool0 = _pool_bytes()
    torch_reserved0 = torch.cuda.memory_reserved()
    for _ in range(3):
        _native.check(lib.ks_synthesize_noalloc(*args))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 >= free0, f"device free memory fell by {free0 - free1} bytes"
    assert _pool_bytes() == pool0
    assert torch.cuda.memory_reserved() == torch_reserved0


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = _native.load()
    g, dcat, datm, _ = _inputs("tiny_500_501")
    big = DeviceGrid(np.linspace(300.0, 1800.0, 2_000_000))  # ~1.7 GB of opacity cubes
    ft = torch.empty(big.n, dtype=torch.float64, device="cuda")
    fc = torch.empty(big.n, dtype=torch.float64, device="cuda")
    st = lib.ks_synthesize_noalloc(C.byref(dcat.rec), C.byref(datm.rec), C.byref(big.rec),
                                   C.byref(make_options()), C.c_void_p(ft.data_ptr()),
                                   C.c_void_p(fc.data_ptr()), None, stream_handle())
    assert st == 3
    assert b"64 MiB" in lib.ks_last_error()
