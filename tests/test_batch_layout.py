"""Batch plan sizing with special lines (CPU only).

ks_batch_workspace_size is host arithmetic over the job records: the records'
pointers are checked for NULL but never dereferenced, so placeholders stand
in for device arrays.  A job's block holds, after its synthesis workspace,
room for its special rows: at most its slice's lines of each class, 4 bytes
each, 256-byte aligned."""

import ctypes as C

from kurucz_py_joss_submission_gb300 import _native

DUMMY = 16   # never dereferenced


def _fill(rec):
    for name, typ in rec._fields_:
        if typ is _native.P:
            setattr(rec, name, DUMMY)
    return rec


def _size(n_lines, counts, first, count):
    L = _native.load(build_if_missing=False)
    lines = _fill(_native.KsLines())
    lines.n_lines = n_lines
    lines.sorted_by_wavelength = 1
    lines.n_hydrogen, lines.n_helium, lines.n_f19 = counts
    atm = _fill(_native.KsAtmos())
    atm.n_layers, atm.n_ion, atm.n_elem, atm.n_edge = 72, 6, 99, 100
    grid = _fill(_native.KsGrid())
    grid.n = 5000
    jobs = (_native.KsJob * 1)()
    jobs[0].atm = C.pointer(atm)
    jobs[0].grid = C.pointer(grid)
    jobs[0].line_first, jobs[0].line_count = first, count
    jobs[0].flux_total = jobs[0].flux_cont = DUMMY
    n = C.c_size_t()
    st = L.ks_batch_workspace_size(C.byref(lines), jobs, 1, None, C.byref(n))
    assert st == _native.KS_OK, L.ks_last_error()
    return n.value


def _rows(n):
    return (4 * n + 255) // 256 * 256


def test_batch_layout_holds_the_special_rows():
    base = _size(1000, (0, 0, 0), 0, 500)
    assert _size(1000, (3, 2, 300), 0, 500) - base == _rows(3 + 2 + 300)
    # a slice of 100 lines holds at most 100 of a class
    base = _size(1000, (0, 0, 0), 200, 100)
    assert _size(1000, (3, 2, 300), 200, 100) - base == _rows(3 + 2 + 100)
    # special lines of the list add nothing to a job without lines
    assert _size(1000, (3, 2, 300), 0, 0) == _size(1000, (0, 0, 0), 0, 0)
