"""Host logic of the batched form (CPU): per-job line slices and size classes."""

import numpy as np

from kurucz_py_joss_submission_gb300 import batch
from kurucz_py_joss_submission_gb300.io.lines import atomic

from _cases import gfall_path


def test_window_slice_equals_filter_by_range():
    cat = atomic.load_catalog(gfall_path("window_500_510"))
    order = np.argsort(cat.wavelength, kind="stable")
    srt = cat.take(order)
    rng = np.random.default_rng(5)
    for _ in range(200):
        a = float(rng.uniform(499.0, 511.0))
        b = a + float(rng.uniform(0.01, 5.0))
        rows = batch.window_slice(srt.wavelength, a, b)
        ref = atomic.filter_by_range(srt, a, b)
        np.testing.assert_array_equal(srt.wavelength[rows], ref.wavelength)


def test_bucket_is_monotone():
    sizes = [1, 500, 1024, 1025, 4096, 4097, 20000, 46245, 537529]
    b = [batch.bucket(n) for n in sizes]
    assert b == sorted(b) and b[0] == 0
