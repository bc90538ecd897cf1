"""Batched form with the special line classes (needs a GPU).

A batch over one shared, wavelength-sorted list holding helium and fort.19
lines (NORMAL, autoionizing, merged continuum): every job, eager and replayed
from the captured graph, equals a standalone synthesis of the same
atmosphere, window and lines bit for bit.  The jobs' special lines are found
at plan time from the list's special rows (each job's a contiguous run of
them) and run between the batch's accumulation and transfer launches, in the
order a single synthesis runs them.

Hydrogen lines go through the C entry point: a job's lines are its slice of
the shared list, and a job whose slice holds a Balmer line equals
ks_synthesize over that slice.  (The Python BatchSynthesizer keeps refusing
lists with hydrogen lines: the reference's window takes hydrogen lines from
a wider margin than the other lines, so its line set is not one slice.)
"""

import numpy as np
import pytest
import torch

from _cases import atm_path, available_cases
from kurucz_py_joss_submission_gb300 import _native, batch, workloads
from kurucz_py_joss_submission_gb300.device import (DeviceAtmosphere, DeviceCatalog, DeviceGrid,
                                                     Synthesizer, make_options)
from kurucz_py_joss_submission_gb300.io import atmosphere as atm_io
from kurucz_py_joss_submission_gb300.io.lines import atomic

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not {"hbeta_486", "hei_447"} <= set(available_cases()),
                                 reason="golden atmospheres missing")]

# (atmosphere, window): fort.19 NORMAL and autoionizing lines, the He I 447.3
# and He II 468.7 nm lines in a 20,000 K model, a window with a merged-
# continuum record, and one without special lines
JOBS = [batch.Job(0, 485.7, 486.5), batch.Job(1, 447.0, 447.5), batch.Job(1, 468.4, 469.0),
        batch.Job(0, 469.8, 470.6), batch.Job(0, 475.0, 475.3), batch.Job(1, 485.9, 486.3)]


def _catalog(tmp_path, hydrogen=True):
    d = workloads.random_atomic_lines(3000, 446.5, 487.0, seed=17)
    n = len(d)
    lo, up = np.zeros(n, np.int32), np.zeros(n, np.int32)
    lo[::10], up[::10] = 3, 5                      # fort.19 NORMAL
    ia = np.arange(75, n, 150)                     # autoionizing
    plain = (d.wavelength_nm > 474.8) & (d.wavelength_nm < 475.5)   # the metal-only job's window
    lo[plain], up[plain] = 0, 0
    ia = ia[~plain[ia]]
    d.n_lower, d.n_upper = lo, up
    tag = np.array([""] * n, dtype=object)
    tag[ia] = "AUT"
    d.tag = tag
    d.log_gamma_rad[ia], d.log_gamma_vdw[ia] = 11.0, 0.3
    d.log_gamma_stark[ia] = np.where(np.arange(ia.size) % 2 == 0, -0.5, 0.3)
    d.log_gf[ia] = np.minimum(d.log_gf[ia], -1.0) - 12.0
    z = np.zeros(2)
    cont = workloads.LineDraw(wavelength_nm=np.array([470.1, 486.0]), log_gf=np.array([-16.0, -15.5]),
                              code=np.full(2, 26.00), e_lower_cm=np.full(2, 1500.0), log_gamma_rad=z + 8.0,
                              log_gamma_stark=z - 5.0, log_gamma_vdw=z - 7.5,
                              labelp=np.array(["CONTINUU"] * 2, dtype=object), xjp=np.array([40.0, 50.0]))
    extra = [workloads.balmer_lines([4])] if hydrogen else []
    d = workloads.merge_lines(d, *extra, workloads.helium_lines(446.5, 487.0), cont)
    p = tmp_path / ("special.gf" if hydrogen else "special_noh.gf")
    workloads.write_gfall(p, d)
    cat = atomic.load_catalog(p)
    return cat.take(np.argsort(cat.wavelength, kind="stable"))


def _single(srt, atms, j, precision):
    sub = atomic.filter_by_range(srt, j.wl_start, j.wl_end)
    g = batch.wavelength_grid(j.wl_start, j.wl_end)
    dcat = DeviceCatalog(sub)
    syn = Synthesizer(dcat, DeviceAtmosphere(atms[j.atmosphere]), DeviceGrid(g), make_options(precision=precision),
                      keep_asynth=False)
    st = syn.run(stats=True)
    torch.cuda.synchronize()
    return syn, st, (dcat.n_hydrogen, dcat.n_helium, dcat.n_f19)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_batch_with_special_lines_equals_single_syntheses(precision, tmp_path):
    srt = _catalog(tmp_path, hydrogen=False)
    atms = [atm_io.load_cached(atm_path("hbeta_486")), atm_io.load_cached(atm_path("hei_447"))]
    cat = DeviceCatalog(srt)
    assert cat.n_hydrogen == 0 and cat.n_helium > 0 and cat.n_f19 > 0
    bs = batch.BatchSynthesizer(cat, atms, JOBS, precision=precision)
    st = bs.run(stats=True)
    assert st["device_flags"] == 0
    bs.capture()
    for f in bs.flux_total + bs.flux_cont:
        f.zero_()
    bs.replay(check=True)
    torch.cuda.synchronize()
    counts = []
    for i, j in enumerate(JOBS):
        syn, one, c = _single(srt, atms, j, precision)
        counts.append(c)
        assert one["device_flags"] == 0
        assert torch.equal(bs.flux_total[i], syn.flux_total), i
        assert torch.equal(bs.flux_cont[i], syn.flux_cont), i
    # the windows cover every class, and one job has no special line
    assert counts[0][2] > 0 and counts[3][2] > 0
    assert counts[1][1] > 0 and counts[2][1] > 0
    assert counts[4] == (0, 0, 0)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_batch_c_entry_with_hydrogen_lines_in_the_slices(precision, tmp_path):
    import ctypes as C

    from kurucz_py_joss_submission_gb300.device import _ptr, stream_handle

    srt = _catalog(tmp_path)
    dcat = DeviceCatalog(srt)
    assert dcat.n_hydrogen == 1
    atms = [DeviceAtmosphere(atm_io.load_cached(atm_path("hbeta_486"))),
            DeviceAtmosphere(atm_io.load_cached(atm_path("hei_447")))]
    wl = np.asarray(srt.wavelength)
    wins = [(0, 485.7, 486.5), (1, 485.9, 486.3), (0, 469.8, 470.6), (1, 447.0, 447.5)]
    grids = [DeviceGrid(batch.wavelength_grid(w0, w1)) for _, w0, w1 in wins]
    slices = [batch.window_slice(wl, w0, w1) for _, w0, w1 in wins]
    ft = [torch.zeros(g.n, dtype=torch.float64, device="cuda") for g in grids]
    fc = [torch.zeros(g.n, dtype=torch.float64, device="cuda") for g in grids]
    jobs = (_native.KsJob * len(wins))()
    for i, (a, _, _) in enumerate(wins):
        jobs[i].atm = C.pointer(atms[a].rec)
        jobs[i].grid = C.pointer(grids[i].rec)
        jobs[i].line_first = slices[i].start
        jobs[i].line_count = slices[i].stop - slices[i].start
        jobs[i].flux_total = ft[i].data_ptr()
        jobs[i].flux_cont = fc[i].data_ptr()
    opts = make_options(precision=precision)
    lib = _native.load()
    size = C.c_size_t()
    _native.check(lib.ks_batch_workspace_size(C.byref(dcat.rec), jobs, len(wins), C.byref(opts), C.byref(size)))
    ws = torch.empty(int(size.value) + 256, dtype=torch.uint8, device="cuda")
    base = (ws.data_ptr() + 255) // 256 * 256
    _native.check(lib.ks_synthesize_batch(C.byref(dcat.rec), jobs, len(wins), C.byref(opts), C.c_void_p(base),
                                          size.value, None, stream_handle()))
    torch.cuda.synchronize()
    n_h = []
    for i, (a, _, _) in enumerate(wins):
        sub = srt.take(np.arange(slices[i].start, slices[i].stop))
        one = DeviceCatalog(sub)
        n_h.append(one.n_hydrogen)
        syn = Synthesizer(one, atms[a], grids[i], make_options(precision=precision), keep_asynth=False)
        st = syn.run(stats=True)
        torch.cuda.synchronize()
        assert st["device_flags"] == 0
        assert torch.equal(ft[i], syn.flux_total), i
        assert torch.equal(fc[i], syn.flux_cont), i
    assert n_h == [1, 1, 0, 0]


def test_batch_rejects_unsorted_special_rows(tmp_path):
    srt = _catalog(tmp_path, hydrogen=False)
    atms = [atm_io.load_cached(atm_path("hbeta_486")), atm_io.load_cached(atm_path("hei_447"))]
    cat = DeviceCatalog(srt)
    assert cat.n_f19 >= 2
    rows = cat.t["f19_rows"]
    rows.copy_(rows.flip(0))   # descending: not the catalog order the plan relies on
    with pytest.raises(_native.KsError, match="ascend"):
        batch.BatchSynthesizer(cat, atms, JOBS[:1], precision="mixed")
