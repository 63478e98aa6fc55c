"""Y-slab decomposition of one stencil field across several owners, with halo-row exchange.

Owner r of W holds rows [r * ny_slab, (r + 1) * ny_slab) of an nx x (W * ny_slab) field: tile r of the
reference's numTiles layout, whose halo pointers name the T rows above and the B rows below each tile
(cuSten/src/struct/custenCreateDestroy2DYp.cu:182-216, periodic formulas: above tile 0 are the field's
last T rows, below the last tile its first B rows). Here each tile lives in its own allocation (one per
process or GPU), so before every Compute each owner receives
    top    = the last T rows of owner r - 1   (wrapping to owner W - 1 for r = 0),
    bottom = the first B rows of owner r + 1  (wrapping to owner 0 for r = W - 1),
and computes its slab with a slab handle (custen_create_slab, `SlabStencil`), which applies the write rules
of tile r of the whole field. Together the slabs give exactly the single-handle result with numTiles = W.

exchange() moves the rows with torch.distributed point-to-point operations: NCCL between GPUs, gloo on the
CPU (the tests). exchange_local() is the same exchange among slabs held by one process.
"""
from __future__ import annotations

import ctypes

from . import F64, HANDLE_BYTES, Stencil, _check, addr, lib


def halo_peers(rank: int, world: int):
    """(owner of the rows above, owner of the rows below) of slab `rank`."""
    return (rank - 1) % world, (rank + 1) % world


def exchange(slab, top, bottom, T: int, B: int, rank: int, world: int, group=None) -> None:
    """Fill `top` (T x nx) with the last T rows of the previous owner and `bottom` (B x nx) with the first B
    rows of the next one. `slab`, `top` and `bottom` are row-major tensors on the device the process group's
    backend serves. Sends carry tag 0 (rows going down) and tag 1 (rows going up), so with two owners, where
    both neighbours are the same process, the two transfers still pair correctly."""
    import torch.distributed as dist
    prev, nxt = halo_peers(rank, world)
    if world == 1:
        if T:
            top.copy_(slab[slab.shape[0] - T:])
        if B:
            bottom.copy_(slab[:B])
        return
    ops = []
    if T:
        ops.append(dist.P2POp(dist.isend, slab[slab.shape[0] - T:].contiguous(), nxt, group, 0))
        ops.append(dist.P2POp(dist.irecv, top, prev, group, 0))
    if B:
        ops.append(dist.P2POp(dist.isend, slab[:B].contiguous(), prev, group, 1))
        ops.append(dist.P2POp(dist.irecv, bottom, nxt, group, 1))
    for req in dist.batch_isend_irecv(ops):
        req.wait()


def exchange_local(slabs, tops, bottoms, T: int, B: int) -> None:
    """The exchange of `exchange` among the slabs of one process (tensors with copy_, any devices)."""
    W = len(slabs)
    for r in range(W):
        prev, nxt = halo_peers(r, W)
        if T:
            tops[r].copy_(slabs[prev][slabs[prev].shape[0] - T:])
        if B:
            bottoms[r].copy_(slabs[nxt][:B])


class SlabStencil(Stencil):
    """A handle over slab `slab` of `num_slabs` (custen_create_slab): tile `slab` of a field of num_slabs
    tiles of ny_slab rows, its halo rows read from `halo_top` / `halo_bottom` (either may be None where the
    variant never reads it). Compute, Swap (which keeps the halo buffers) and Destroy as for `Stencil`."""

    def __init__(self, variant: int, nx: int, ny_slab: int, slab: int, num_slabs: int, out, inp, halo_top,
                 halo_bottom, coef, *, H=1, L=0, R=0, V=1, T=0, B=0, block_x=32, block_y=8, dtype=F64, device=0,
                 ncoef=None, func=None):
        self.variant, self.dtype = variant, dtype
        self.nx, self.ny = nx, ny_slab
        self.slab, self.num_slabs = slab, num_slabs
        self.handle = ctypes.create_string_buffer(HANDLE_BYTES)
        if ncoef is None:
            ncoef = H * V
        self._alive = False
        _check(lib().custen_create_slab(self.handle, variant, dtype, device, slab, num_slabs, nx, ny_slab, block_x,
                                        block_y, addr(out), addr(inp), addr(halo_top), addr(halo_bottom), addr(coef),
                                        H, L, R, V, T, B, ncoef, addr(func)))
        self._alive = True
