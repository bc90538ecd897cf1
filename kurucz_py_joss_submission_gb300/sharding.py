"""Synthesis of one spectrum sharded over GPUs, one process per GPU.

Every stage before the transfer works layer by layer -- continuum
(synthe_py/physics/continuum.py:73-303), TRANSP (line_opacity.py:56-184) and
ASYNTH (line_opacity.py:946-1340) loop over depths independently -- and the
transfer works wavelength by wavelength (engine/radiative.py:282-494).  So
rank r takes a contiguous block of layers through ``ks_opacity``, one
all-to-all exchange turns its ``[layers, lambda]`` cubes (ASYNTH and the two
continuum opacities) into ``[all layers, lambda slice]`` cubes, and rank r
solves its wavelength slice with ``ks_transfer_opacity``.  No stage is
repeated across ranks, and the spectrum stitched from the slices is
bit-identical to the unsharded ``ks_synthesize`` result: each layer's
accumulation and each wavelength's transfer run the same code on the same
numbers.

The exchange is ``torch.distributed.all_to_all_single`` (NCCL between GPUs,
gloo for the CPU tests); ``emulate`` runs all ranks in one process on one GPU
with the same packing, for parity tests without a second GPU.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import replace
from typing import List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _native
from .device import (DeviceAtmosphere, DeviceCatalog, DeviceGrid, _ptr, make_options,
                     stream_handle)
from .io.atmosphere import AtmosphereModel

Block = Tuple[int, int]


def blocks(n: int, parts: int) -> List[Block]:
    """``parts`` contiguous ranges covering ``[0, n)``, sizes differing by at most one."""
    if parts < 1:
        raise ValueError("parts must be >= 1")
    base, extra = divmod(n, parts)
    out, start = [], 0
    for p in range(parts):
        size = base + (1 if p < extra else 0)
        out.append((start, start + size))
        start += size
    return out


_LAYER_FIELDS = ("depth", "temperature", "gas_pressure", "electron_density", "mass_density",
                 "turbulent_velocity", "hckt", "xnf_h", "xnf_he1", "xnf_h2", "population_per_ion",
                 "doppler_per_ion", "continuum_abs_coeff", "continuum_scat_coeff")


def slice_layers(atm: AtmosphereModel, d0: int, d1: int) -> AtmosphereModel:
    """The layers ``[d0, d1)`` of an atmosphere (per-layer arrays sliced on
    their first axis; the continuum edge tables are shared)."""
    kw = {}
    for name in _LAYER_FIELDS:
        v = getattr(atm, name)
        kw[name] = None if v is None else np.ascontiguousarray(np.asarray(v)[d0:d1])
    return replace(atm, **kw)


def pack(cubes: Sequence[torch.Tensor], slices: Sequence[Block]) -> Tuple[torch.Tensor, List[int]]:
    """Send buffer of the all-to-all: for each destination rank k in order,
    every cube's columns ``slices[k]`` (rows of this rank's layer block),
    flattened.  Returns the buffer and the per-destination element counts."""
    rows = cubes[0].shape[0]
    parts, sizes = [], []
    for j0, j1 in slices:
        chunk = [c[:, j0:j1].reshape(-1) for c in cubes]
        parts.extend(chunk)
        sizes.append(len(cubes) * rows * (j1 - j0))
    return torch.cat(parts) if parts else cubes[0].new_empty(0), sizes


def unpack(buf: torch.Tensor, depth_blocks: Sequence[Block], width: int, ncubes: int) -> List[torch.Tensor]:
    """Receive buffer of the all-to-all (the chunks from each source rank in
    rank order) -> ``ncubes`` cubes ``[all layers, width]``."""
    out = [[] for _ in range(ncubes)]
    off = 0
    for d0, d1 in depth_blocks:
        rows = d1 - d0
        for c in range(ncubes):
            n = rows * width
            out[c].append(buf[off:off + n].view(rows, width))
            off += n
    return [torch.cat(parts, dim=0).contiguous() for parts in out]


def exchange(cubes: Sequence[torch.Tensor], depth_blocks: Sequence[Block], slices: Sequence[Block],
             rank: int, group=None) -> List[torch.Tensor]:
    """This rank's ``[layers of its block, lambda]`` cubes -> ``[all layers,
    its lambda slice]`` cubes, through one ``all_to_all_single``."""
    import torch.distributed as dist

    send, send_sizes = pack(cubes, slices)
    j0, j1 = slices[rank]
    width = j1 - j0
    recv_sizes = [len(cubes) * (d1 - d0) * width for d0, d1 in depth_blocks]
    recv = send.new_empty(sum(recv_sizes))
    dist.all_to_all_single(recv, send, output_split_sizes=recv_sizes, input_split_sizes=send_sizes,
                           group=group)
    return unpack(recv, depth_blocks, width, len(cubes))


class ShardRank:
    """One rank of a sharded synthesis: its layer block through ks_opacity,
    its wavelength slice through ks_transfer_opacity."""

    def __init__(self, catalog: DeviceCatalog, atm: AtmosphereModel, wavelength: np.ndarray,
                 grid_origin: Optional[float], rank: int, world: int, options=None, device="cuda"):
        self.lib = _native.load()
        self.rank, self.world = rank, world
        self.options = options or make_options()
        self.fp64 = self.options.precision == _native.KS_PREC_FP64
        wavelength = np.ascontiguousarray(wavelength, dtype=np.float64)
        n, L = wavelength.size, atm.layers
        if not 1 <= world <= min(L, n):
            raise ValueError(f"world size {world}: needs 1 <= world <= min(layers {L}, wavelengths {n})")
        self.n, self.L = n, L
        self.depth_blocks = blocks(L, world)
        self.slices = blocks(n, world)
        d0, d1 = self.depth_blocks[rank]
        j0, j1 = self.slices[rank]
        origin = float(grid_origin if grid_origin is not None else (wavelength[0] if n else 0.0))
        self.catalog = catalog
        self.atm_block = DeviceAtmosphere(slice_layers(atm, d0, d1), device=device)
        self.atm_full = DeviceAtmosphere(atm, device=device)
        self.grid = DeviceGrid(wavelength, origin, device=device)
        self.grid_slice = DeviceGrid(wavelength[j0:j1], origin, device=device)
        dev = self.grid.wavelength.device
        ws = C.c_size_t()
        _native.check(self.lib.ks_workspace_size(catalog.n_lines, d1 - d0, n, C.byref(self.options),
                                                 C.byref(ws)))
        self.workspace_bytes = int(ws.value)
        self.workspace = torch.empty(self.workspace_bytes, dtype=torch.uint8, device=dev)
        dt = torch.float64 if self.fp64 else torch.float32
        self.cubes = [torch.empty((d1 - d0, n), dtype=dt, device=dev) for _ in range(3)]  # asynth, abs, scat
        self.flux_total = torch.empty(j1 - j0, dtype=torch.float64, device=dev)
        self.flux_cont = torch.empty(j1 - j0, dtype=torch.float64, device=dev)

    def opacity(self, stats: bool = False, stream=None):
        st = _native.KsStats()
        _native.check(self.lib.ks_opacity(
            C.byref(self.catalog.rec), C.byref(self.atm_block.rec), C.byref(self.grid.rec),
            C.byref(self.options), _ptr(self.workspace), self.workspace_bytes,
            _ptr(self.cubes[0]), _ptr(self.cubes[1]), _ptr(self.cubes[2]),
            C.byref(st) if stats else None, stream_handle(stream)))
        return st.as_dict() if stats else None

    def transfer(self, slab: Sequence[torch.Tensor], stats: bool = False, stream=None):
        asy, cab, csc = slab
        st = _native.KsStats()
        _native.check(self.lib.ks_transfer_opacity(
            C.byref(self.atm_full.rec), C.byref(self.grid_slice.rec), C.byref(self.options),
            _ptr(cab), _ptr(csc), _ptr(asy), _ptr(self.flux_total), _ptr(self.flux_cont),
            C.byref(st) if stats else None, stream_handle(stream)))
        return st.as_dict() if stats else None

    def run(self, group=None, stats: bool = False):
        """Opacity, exchange, transfer.  With ``stats`` the counters are
        summed over ranks (evaluations, valid pairs, iterations)."""
        s1 = self.opacity(stats)
        slab = exchange(self.cubes, self.depth_blocks, self.slices, self.rank, group)
        s2 = self.transfer(slab, stats)
        if not stats:
            return None
        import torch.distributed as dist

        v = torch.tensor([s1["valid_pairs"], s1["evaluations"], s2["iterations"], s2["maxj_wavelengths"]],
                         dtype=torch.int64, device=self.flux_total.device)
        dist.all_reduce(v, group=group)
        return {"valid_pairs": int(v[0]), "evaluations": int(v[1]), "iterations": int(v[2]),
                "maxj_wavelengths": int(v[3]),
                "kernel_launches": s1["kernel_launches"] + s2["kernel_launches"]}


def gather_flux(part: torch.Tensor, slices: Sequence[Block], group=None) -> torch.Tensor:
    """Concatenate every rank's wavelength slice (all ranks receive it)."""
    import torch.distributed as dist

    width = max(j1 - j0 for j0, j1 in slices)
    padded = part.new_zeros(width)
    padded[: part.numel()] = part
    bufs = [part.new_empty(width) for _ in slices]
    dist.all_gather(bufs, padded, group=group)
    return torch.cat([b[: j1 - j0] for b, (j0, j1) in zip(bufs, slices)])


def emulate(catalog: DeviceCatalog, atm: AtmosphereModel, wavelength: np.ndarray,
            grid_origin: Optional[float], world: int, options=None, device="cuda"):
    """All ranks of a ``world``-way sharded run in this process, on one GPU:
    the same ks_opacity / ks_transfer_opacity calls and the same packing,
    with the all-to-all done by slicing the send buffers.  Returns the
    stitched (flux_total, flux_cont) and the summed evaluation count."""
    ranks = [ShardRank(catalog, atm, wavelength, grid_origin, r, world, options, device)
             for r in range(world)]
    evals = 0
    sends = []
    for rk in ranks:
        evals += rk.opacity(stats=True)["evaluations"]
        sends.append(pack(rk.cubes, rk.slices))
    ft, fc = [], []
    for k, rk in enumerate(ranks):
        j0, j1 = rk.slices[k]
        chunks = []
        for buf, sizes in sends:
            off = sum(sizes[:k])
            chunks.append(buf[off:off + sizes[k]])
        slab = unpack(torch.cat(chunks), rk.depth_blocks, j1 - j0, 3)
        rk.transfer(slab)
        ft.append(rk.flux_total)
        fc.append(rk.flux_cont)
    return torch.cat(ft), torch.cat(fc), evals
