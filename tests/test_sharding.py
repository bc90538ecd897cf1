"""Host logic of the depth-sharded synthesis (CPU, gloo, world size 2 and 3)."""

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from kurucz_py_joss_submission_gb300 import sharding
from kurucz_py_joss_submission_gb300.io import atmosphere as atm_io

from _cases import atm_path


def test_blocks_cover_and_balance():
    for n in (1, 5, 72, 537529):
        for parts in range(1, min(n, 9) + 1):
            b = sharding.blocks(n, parts)
            assert b[0][0] == 0 and b[-1][1] == n
            assert all(b[i][1] == b[i + 1][0] for i in range(parts - 1))
            sizes = [e - s for s, e in b]
            assert max(sizes) - min(sizes) <= 1


def test_slice_layers_keeps_edge_tables():
    atm = atm_io.load_cached(atm_path("tiny_500_501"))
    sub = sharding.slice_layers(atm, 10, 30)
    assert sub.layers == 20
    np.testing.assert_array_equal(sub.temperature, atm.temperature[10:30])
    np.testing.assert_array_equal(sub.population_per_ion, atm.population_per_ion[10:30])
    np.testing.assert_array_equal(sub.continuum_abs_coeff, atm.continuum_abs_coeff[10:30])
    np.testing.assert_array_equal(sub.continuum_wledge, atm.continuum_wledge)


def _cube(rows, n, k):
    d = torch.arange(rows[0], rows[1], dtype=torch.float64)[:, None]
    j = torch.arange(n, dtype=torch.float64)[None, :]
    return (k + 1) * (1000.0 * d + j)


def _worker(rank, world, port, L, n, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        db = sharding.blocks(L, world)
        sl = sharding.blocks(n, world)
        cubes = [_cube(db[rank], n, k) for k in range(3)]
        slab = sharding.exchange(cubes, db, sl, rank)
        j0, j1 = sl[rank]
        ok = all(torch.equal(slab[k], _cube((0, L), n, k)[:, j0:j1]) for k in range(3))
        part = torch.arange(j0, j1, dtype=torch.float64) * 0.5
        full = sharding.gather_flux(part, sl)
        ok = ok and torch.equal(full, torch.arange(n, dtype=torch.float64) * 0.5)
        q.put((rank, bool(ok)))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world,L,n", [(2, 72, 101), (3, 7, 10), (2, 5, 2)])
def test_exchange_and_gather_gloo(world, L, n):
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    mp.start_processes(_worker, args=(world, _free_port(), L, n, q), nprocs=world, join=True,
                       start_method="spawn")
    res = sorted(q.get() for _ in range(world))
    assert res == [(r, True) for r in range(world)]


def test_pack_unpack_roundtrip_single_process():
    L, n, world = 9, 13, 3
    db, sl = sharding.blocks(L, world), sharding.blocks(n, world)
    sends = [sharding.pack([_cube(db[r], n, k) for k in range(3)], sl) for r in range(world)]
    for k in range(world):
        chunks = []
        for buf, sizes in sends:
            off = sum(sizes[:k])
            chunks.append(buf[off:off + sizes[k]])
        j0, j1 = sl[k]
        slab = sharding.unpack(torch.cat(chunks), db, j1 - j0, 3)
        for c in range(3):
            assert torch.equal(slab[c], _cube((0, L), n, c)[:, j0:j1])
