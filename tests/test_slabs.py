"""Y-slab decomposition of one field across owners with halo-row exchange (custen_gb300.slabs).

CPU (gloo, world sizes 2 and 3, one process per owner): each owner holds only its slab, receives its halo
rows through slabs.exchange, and computes its rows with the oracle from nothing but its slab and the
received rows; the owners' rows together must equal the single-field oracle result with numTiles = world,
bit for bit. This checks which rows travel where (periodic wrap at both ends, the non-periodic edges).

GPU (one process emulating four owners on one device, exchange_local): slab handles
(custen_create_slab) against one ordinary handle with numTiles = 4 and against the oracle, bit for bit,
for the twelve variants, FP64 and FP32, and a Compute / Swap / exchange / Compute sequence. Every call of
this suite gets one GPU: the NCCL data plane of exchange() is not run on hardware here.
"""
import os
import socket

import numpy as np
import pytest

import custen_gb300 as cs
import oracle
from custen_gb300 import slabs
from custen_gb300.inputs import field, sentinel
from tests.helpers import weights_for

FUN_IDS = {0: 1, 1: 3, 2: 5}   # the c^3 - c device functions (window: X / Y 5-point, XY any)


def _geometry(variant):
    d = 0 if variant < 4 else (1 if variant < 8 else 2)
    if variant in (cs.XPFUN, cs.XNPFUN, cs.YPFUN, cs.YNPFUN, cs.XYPFUN, cs.XYNPFUN):
        geom = {0: (5, 2, 2, 1, 0, 0), 1: (1, 0, 0, 5, 2, 2), 2: (4, 2, 1, 3, 1, 1)}[d]
        H, V = geom[0], geom[3]
        ncoef = {0: 5, 1: 5, 2: H * V}[d]
        return geom, FUN_IDS[d], ncoef
    geom = {0: (4, 2, 1, 1, 0, 0), 1: (1, 0, 0, 4, 1, 2), 2: (4, 1, 2, 4, 2, 1)}[d]
    return geom, -1, geom[0] * geom[3]


def _coef(variant, geom, fun_id, ncoef, dtype=np.float64):
    if fun_id >= 0:
        return np.random.default_rng(60 + variant).uniform(-1, 1, ncoef).astype(dtype)
    return weights_for(variant, geom[0], geom[3], 60 + variant, dtype)


def rank_rows_via_oracle(variant, slab_in, top, bottom, rank, world, geom, coef, fun_id, bx, by):
    """The rows of slab `rank` computed by the oracle from the slab and its received halo rows only: every
    other row of the input is NaN, and the halo rows sit where the tile's halo pointers name them."""
    H, L, R, V, T, B = geom
    nys, nx = slab_in.shape
    ny = world * nys
    inp = np.full((ny, nx), np.nan)
    inp[rank * nys:(rank + 1) * nys] = slab_in
    halo = np.full((ny, nx), np.nan)
    for k in range(T):
        halo[(rank * nys - T + k) % ny] = top[k]
    for k in range(B):
        halo[((rank + 1) * nys + k) % ny] = bottom[k]
    out = sentinel(nx, ny)
    oracle.stencil(variant, out, inp, coef, num_tiles=world, block_x=bx, block_y=by, H=H, L=L, R=R, V=V, T=T, B=B,
                   fun_id=fun_id, halo_src=halo)
    return out[rank * nys:(rank + 1) * nys]


VARIANTS_Y = [cs.YP, cs.YNP, cs.YPFUN, cs.YNPFUN, cs.XYP, cs.XYNP, cs.XYPFUN, cs.XYNPFUN]
NX, NYS, BX, BY = 32, 16, 8, 4


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _owner(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        full = field(NX, world * NYS, 5)
        mine = torch.tensor(full[rank * NYS:(rank + 1) * NYS])   # this owner's slab; the rest is not used
        results = {}
        for variant in VARIANTS_Y:
            geom, fun_id, ncoef = _geometry(variant)
            T, B = geom[4], geom[5]
            top, bottom = torch.zeros((T, NX), dtype=torch.float64), torch.zeros((B, NX), dtype=torch.float64)
            slabs.exchange(mine, top, bottom, T, B, rank, world)
            coef = _coef(variant, geom, fun_id, ncoef)
            results[variant] = rank_rows_via_oracle(variant, mine.numpy(), top.numpy(), bottom.numpy(), rank, world,
                                                    geom, coef, fun_id, BX, BY)
        q.put((rank, results))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_gloo_owners_equal_single_field(world):
    import torch.multiprocessing as mp
    oracle.build()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_owner, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=300) for _ in range(world))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    full = field(NX, world * NYS, 5)
    for variant in VARIANTS_Y:
        geom, fun_id, ncoef = _geometry(variant)
        H, L, R, V, T, B = geom
        ref = sentinel(NX, world * NYS)
        oracle.stencil(variant, ref, full, _coef(variant, geom, fun_id, ncoef), num_tiles=world, block_x=BX,
                       block_y=BY, H=H, L=L, R=R, V=V, T=T, B=B, fun_id=fun_id)
        assembled = np.concatenate([got[r][variant] for r in range(world)])
        assert assembled.tobytes() == ref.tobytes(), cs.VARIANT_NAMES[variant]


def test_local_exchange_rows():
    """exchange_local fills each slab's halos with its neighbours' edge rows, wrapping at both ends."""
    import torch
    W, T, B = 4, 2, 3
    full = torch.arange(W * 6 * 5, dtype=torch.float64).reshape(W * 6, 5)
    parts = list(full.split(6))
    tops = [torch.empty(T, 5, dtype=torch.float64) for _ in range(W)]
    bots = [torch.empty(B, 5, dtype=torch.float64) for _ in range(W)]
    slabs.exchange_local(parts, tops, bots, T, B)
    for r in range(W):
        assert torch.equal(tops[r], full[[(r * 6 - T + k) % (W * 6) for k in range(T)]])
        assert torch.equal(bots[r], full[[((r + 1) * 6 + k) % (W * 6) for k in range(B)]])


def _run_slabs_gpu(variant, dtype, W=4, nx=128, nys=64, bx=32, by=8, steps=1):
    import torch
    geom, fun_id, ncoef = _geometry(variant)
    H, L, R, V, T, B = geom
    dev = torch.device("cuda", 0)
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    cdt = cs.F64 if dtype == np.float64 else cs.F32
    ny = W * nys
    full = field(nx, ny, 9, dtype)
    coef = _coef(variant, geom, fun_id, ncoef, dtype)
    pre = sentinel(nx, ny, dtype)
    func = cs.builtin_function(fun_id, cdt) if fun_id >= 0 else None
    wt = torch.tensor(coef, device=dev)
    # W owners on one device
    ins = [torch.tensor(full[r * nys:(r + 1) * nys], device=dev) for r in range(W)]
    outs = [torch.tensor(pre[r * nys:(r + 1) * nys], device=dev) for r in range(W)]
    tops = [torch.zeros((max(T, 1), nx), device=dev, dtype=tdt) for _ in range(W)]
    bots = [torch.zeros((max(B, 1), nx), device=dev, dtype=tdt) for _ in range(W)]
    hs = [slabs.SlabStencil(variant, nx, nys, r, W, outs[r], ins[r], tops[r] if T else None, bots[r] if B else None,
                            wt, H=H, L=L, R=R, V=V, T=T, B=B, block_x=bx, block_y=by, dtype=cdt, ncoef=ncoef,
                            func=func) for r in range(W)]
    # one ordinary handle with numTiles = W over the whole field
    d_in, d_out = torch.tensor(full, device=dev), torch.tensor(pre, device=dev)
    single = cs.Stencil(variant, nx, ny, d_out, d_in, wt, H=H, L=L, R=R, V=V, T=T, B=B, num_tiles=W, block_x=bx,
                        block_y=by, dtype=cdt, ncoef=ncoef, func=func)
    cur_in, cur_out = ins, outs
    for step in range(steps):
        slabs.exchange_local(cur_in, tops, bots, T, B)
        for h in hs:
            h.compute()
        single.compute()
        if step + 1 < steps:
            for r, h in enumerate(hs):
                h.swap(cur_out[r])
            single.swap(d_out)
            cur_in, cur_out = cur_out, cur_in
            d_in, d_out = d_out, d_in
    torch.cuda.synchronize(dev)
    got = torch.cat(cur_out).cpu().numpy()
    ref_single = d_out.cpu().numpy()
    for h in hs:
        h.destroy()
    single.destroy()
    return got, ref_single, full, coef, geom, fun_id, pre


@pytest.mark.gpu
@pytest.mark.parametrize("variant", list(range(12)), ids=cs.VARIANT_NAMES)
@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
def test_slab_handles_equal_single_handle(gpu, variant, dtype):
    got, ref_single, full, coef, geom, fun_id, pre = _run_slabs_gpu(variant, dtype)
    H, L, R, V, T, B = geom
    assert got.tobytes() == ref_single.tobytes(), "slabs differ from the numTiles handle"
    ref = pre.copy()
    st = oracle.stencil(variant, ref, full, coef, num_tiles=4, block_x=32, block_y=8, H=H, L=L, R=R, V=V, T=T, B=B,
                        fun_id=fun_id)
    w = st == 1
    assert np.array_equal(got[w], ref[w])
    assert np.array_equal(got[~w], pre[~w])
    assert cs.device_error() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [cs.YP, cs.XYNP, cs.XYPFUN])
def test_slab_handles_swap_sequence(gpu, variant):
    """Compute, Swap, exchange the new input's halos, Compute: equal to the numTiles handle doing the same."""
    got, ref_single, *_ = _run_slabs_gpu(variant, np.float64, steps=3)
    assert got.tobytes() == ref_single.tobytes()


@pytest.mark.gpu
def test_slab_handle_argument_errors(gpu):
    import torch
    dev = torch.device("cuda", 0)
    a = torch.zeros((64, 64), device=dev, dtype=torch.float64)
    w = torch.ones(5, device=dev, dtype=torch.float64)
    with pytest.raises(cs.CustenError, match="halo_top is NULL"):
        slabs.SlabStencil(cs.YP, 64, 64, 1, 2, a, a, None, a, w, V=5, T=2, B=2)
    with pytest.raises(cs.CustenError, match="index must lie"):
        slabs.SlabStencil(cs.YP, 64, 64, 2, 2, a, a, a, a, w, V=5, T=2, B=2)
