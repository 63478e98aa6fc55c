"""Parity of the sm_103a stencil kernels with the oracle (GPU).

Every written point must be bit-identical to the oracle's FMA chain; every point the reference leaves
untouched must keep the sentinel it was pre-filled with; points the reference writes from shared
memory it never loaded (oracle status 2) are left untouched by this library.
"""
import numpy as np
import pytest

import custen_gb300 as cs
import oracle
from custen_gb300.buffers import DeviceBuffer, HostBuffer
from custen_gb300.inputs import field, sentinel
from tests.helpers import weights_for

pytestmark = pytest.mark.gpu

FUN_IDS = {0: (0, 1), 1: (2, 3), 2: (4, 5)}  # shipped device functions per direction


def geometry(variant, kind):
    """(H, L, R, V, T, B) for a direction and a halo shape."""
    d = 0 if variant < 4 else (1 if variant < 8 else 2)
    shapes = {
        0: {"sym": (5, 2, 2, 1, 0, 0), "asym": (5, 3, 1, 1, 0, 0), "small": (3, 1, 1, 1, 0, 0)},
        1: {"sym": (1, 0, 0, 5, 2, 2), "asym": (1, 0, 0, 5, 1, 3), "small": (1, 0, 0, 3, 1, 1)},
        2: {"sym": (5, 2, 2, 5, 2, 2), "asym": (4, 2, 1, 3, 1, 1), "small": (3, 1, 1, 3, 1, 1)},
    }
    return shapes[d][kind]


def run_both(variant, nx, ny, tiles, bx, by, geom, dtype=np.float64, fun_id=-1, seed=0, managed=False,
             offload=cs.DEVICE, mem=None, config=None):
    """mem: "device" (default), "managed", "pinned" (cudaMallocHost) or "pageable" (numpy memory)."""
    mem = mem or ("managed" if managed else "device")
    H, L, R, V, T, B = geom
    inp = field(nx, ny, seed, dtype)
    fun = fun_id >= 0
    if fun:
        ncoef = {0: 1, 1: 5, 2: 9, 3: 5, 4: H * V, 5: H * V}[fun_id]
        coef = np.random.default_rng(50 + seed).uniform(-1, 1, ncoef).astype(dtype)
    else:
        coef = weights_for(variant, H, V, seed, dtype)
        ncoef = coef.size
    pre = sentinel(nx, ny, dtype)
    ref = pre.copy()
    st = oracle.stencil(variant, ref, inp, coef, num_tiles=tiles, block_x=bx, block_y=by, H=H, L=L, R=R, V=V, T=T,
                        B=B, fun_id=fun_id)

    dt = cs.F64 if dtype == np.float64 else cs.F32
    if mem in ("device", "managed"):
        d_in = DeviceBuffer.from_array(inp, mem == "managed")
        d_out = DeviceBuffer.from_array(pre, mem == "managed")
        d_c = DeviceBuffer.from_array(coef, mem == "managed")
        ptrs = (d_out.ptr, d_in.ptr, d_c.ptr)
    elif mem == "pinned":
        d_in, d_out, d_c = HostBuffer.from_array(inp), HostBuffer.from_array(pre), HostBuffer.from_array(coef)
        ptrs = (d_out.ptr, d_in.ptr, d_c.ptr)
    else:
        d_in, d_out, d_c = inp.copy(), pre.copy(), coef.copy()
        ptrs = (d_out.ctypes.data, d_in.ctypes.data, d_c.ctypes.data)
    func = cs.builtin_function(fun_id, dt) if fun else None
    s = cs.Stencil(variant, nx, ny, ptrs[0], ptrs[1], ptrs[2], H=H, L=L, R=R, V=V, T=T, B=B, num_tiles=tiles,
                   block_x=bx, block_y=by, dtype=dt, ncoef=ncoef, func=func)
    if config is not None:
        s.set_config(config)
    s.compute(offload)
    cs._check(cs.lib().custen_device_synchronize())
    if mem == "device":
        got = d_out.download((ny, nx), dtype)
    elif mem == "pageable":
        got = d_out.copy()
    else:
        got = d_out.view((ny, nx), dtype).copy()
    s.destroy()
    return got, ref, st, pre


def check(got, ref, st, pre):
    w = st == 1
    bad = w & ~((got == ref) | (np.isnan(got) & np.isnan(ref)))
    assert not bad.any(), f"{bad.sum()} written points differ; first at {np.argwhere(bad)[:3].tolist()}"
    keep = st != 1
    assert np.array_equal(got[keep], pre[keep]), "points the reference leaves untouched were modified"


VARIANTS = list(range(12))


@pytest.mark.parametrize("variant", VARIANTS, ids=cs.VARIANT_NAMES)
@pytest.mark.parametrize("tiles", [1, 2, 4])
@pytest.mark.parametrize("kind", ["sym", "asym"])
def test_parity_f64(gpu, variant, tiles, kind):
    geom = geometry(variant, kind)
    d = 0 if variant < 4 else (1 if variant < 8 else 2)
    fun = variant in (cs.XPFUN, cs.XNPFUN, cs.YPFUN, cs.YNPFUN, cs.XYPFUN, cs.XYNPFUN)
    fun_id = -1
    if fun:
        fun_id = FUN_IDS[d][1]           # the (c^3 - c) functions reach 2 points
        if d == 1:
            geom = (1, 0, 0, 5, 2, 2)
        elif d == 0:
            geom = (5, 2, 2, 1, 0, 0)
    nx, ny = (96, 64) if d != 1 else (48, 128)
    got, ref, st, pre = run_both(variant, nx, ny, tiles, 32 if d != 1 else 16, 8, geom, fun_id=fun_id,
                                 seed=variant * 7 + tiles)
    check(got, ref, st, pre)


@pytest.mark.parametrize("variant", VARIANTS, ids=cs.VARIANT_NAMES)
def test_parity_f32(gpu, variant):
    d = 0 if variant < 4 else (1 if variant < 8 else 2)
    fun = variant in (cs.XPFUN, cs.XNPFUN, cs.YPFUN, cs.YNPFUN, cs.XYPFUN, cs.XYNPFUN)
    geom = geometry(variant, "sym")
    fun_id = FUN_IDS[d][1] if fun else -1
    nx, ny = (128, 64) if d != 1 else (64, 128)
    got, ref, st, pre = run_both(variant, nx, ny, 2, 32, 8, geom, dtype=np.float32, fun_id=fun_id, seed=variant)
    check(got, ref, st, pre)


@pytest.mark.parametrize("variant", [cs.XP, cs.XNP, cs.YP, cs.YNP, cs.XYP, cs.XYNP])
@pytest.mark.parametrize("tiles", [1, 3])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_parity_radius_4(gpu, variant, tiles, dtype):
    """Radius-4 windows (X 9-point, Y 9-point, XY 9 x 9), numTiles 1 and 3."""
    d = 0 if variant < 4 else (1 if variant < 8 else 2)
    geom = {0: (9, 4, 4, 1, 0, 0), 1: (1, 0, 0, 9, 4, 4), 2: (9, 4, 4, 9, 4, 4)}[d]
    got, ref, st, pre = run_both(variant, 96, 96, tiles, 32, 8, geom, dtype=dtype, seed=41 + variant + tiles)
    check(got, ref, st, pre)


@pytest.mark.parametrize("variant", [cs.XP, cs.XNP, cs.YP, cs.YNP, cs.XYP, cs.XYNP])
def test_parity_unaligned_rows(gpu, variant):
    """nx = 98 doubles: rows are not 16-byte aligned, the scalar staging/store path runs."""
    d = 0 if variant < 4 else (1 if variant < 8 else 2)
    got, ref, st, pre = run_both(variant, 98, 56, 2, 14, 4, geometry(variant, "small"), seed=11)
    check(got, ref, st, pre)


@pytest.mark.parametrize("variant", [cs.XPFUN, cs.YPFUN, cs.XYPFUN, cs.XNPFUN, cs.YNPFUN, cs.XYNPFUN])
def test_parity_reference_example_functions(gpu, variant):
    """The example user functions: X 3-point (id 0), Y 9-point (id 2), XY weighted window (id 4)."""
    d = 0 if variant < 4 else (1 if variant < 8 else 2)
    geom = {0: (3, 1, 1, 1, 0, 0), 1: (1, 0, 0, 9, 4, 4), 2: (3, 1, 1, 3, 1, 1)}[d]
    fun_id = FUN_IDS[d][0]
    nx, ny = (64, 64) if d != 1 else (32, 128)
    got, ref, st, pre = run_both(variant, nx, ny, 2, 16 if d != 1 else 8, 8, geom, fun_id=fun_id, seed=3)
    check(got, ref, st, pre)


@pytest.mark.parametrize("variant", [cs.XPFUN, cs.XNPFUN, cs.YPFUN, cs.YNPFUN, cs.XYPFUN, cs.XYNPFUN])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_fused_and_indirect_fun_paths_agree(gpu, variant, dtype):
    """The library's c^3 - c functions run fused (cube once per value, then weights) by default and through
    the indirect call when fusion is off: both give the oracle's result and are bitwise identical."""
    d = 0 if variant < 4 else (1 if variant < 8 else 2)
    geom = {0: (5, 2, 2, 1, 0, 0), 1: (1, 0, 0, 5, 2, 2), 2: (3, 1, 1, 3, 1, 1)}[d]
    nx, ny = (128, 64) if d != 1 else (64, 128)
    got_fused, ref, st, pre = run_both(variant, nx, ny, 2, 32 if d != 1 else 16, 8, geom, dtype=dtype,
                                       fun_id=FUN_IDS[d][1], seed=17 + variant)
    check(got_fused, ref, st, pre)
    cs.set_fun_fusion(False)
    try:
        got_call, *_ = run_both(variant, nx, ny, 2, 32 if d != 1 else 16, 8, geom, dtype=dtype,
                                fun_id=FUN_IDS[d][1], seed=17 + variant)
    finally:
        cs.set_fun_fusion(True)
    check(got_call, ref, st, pre)
    assert got_fused.tobytes() == got_call.tobytes()


@pytest.mark.parametrize("variant", [cs.XP, cs.YNP, cs.XYP, cs.XYNPFUN])
def test_managed_memory_tile_streaming(gpu, variant):
    """Managed memory, numTiles = 4, HOST offload: tiles stream through the GPU and come back."""
    d = 0 if variant < 4 else (1 if variant < 8 else 2)
    fun_id = FUN_IDS[d][1] if variant == cs.XYNPFUN else -1
    got, ref, st, pre = run_both(variant, 64, 128, 4, 16, 8, geometry(variant, "sym"), fun_id=fun_id, seed=5,
                                 managed=True, offload=cs.HOST)
    check(got, ref, st, pre)


@pytest.fixture
def small_chunks():
    """Host-resident fields stream in chunks of a few rows, so a tile spans several chunks and the
    staging slots are reused within one Compute."""
    cs.set_stage_chunk_bytes(4096)
    yield
    cs.set_stage_chunk_bytes(0)


@pytest.mark.parametrize("variant", VARIANTS, ids=cs.VARIANT_NAMES)
@pytest.mark.parametrize("tiles", [1, 4])
@pytest.mark.parametrize("mem", ["pinned", "pageable"])
def test_host_memory_streaming(gpu, small_chunks, variant, tiles, mem):
    """Fields in pinned or pageable host memory, HOST offload: rows stream through the device staging
    slots (several chunks per tile, halos across chunk and tile borders) and every written point is
    bit-identical to the oracle; the untouched border keeps its values."""
    d = 0 if variant < 4 else (1 if variant < 8 else 2)
    fun = variant in (cs.XPFUN, cs.XNPFUN, cs.YPFUN, cs.YNPFUN, cs.XYPFUN, cs.XYNPFUN)
    geom = geometry(variant, "asym")
    fun_id = -1
    if fun:
        fun_id = FUN_IDS[d][1]
        geom = {0: (5, 2, 2, 1, 0, 0), 1: (1, 0, 0, 5, 2, 2), 2: (5, 2, 2, 5, 2, 2)}[d]
    h2d0, d2h0 = cs.transfer_bytes()
    nx, ny = 64, 256
    got, ref, st, pre = run_both(variant, nx, ny, tiles, 16, 8, geom, fun_id=fun_id, seed=31 + variant, mem=mem,
                                 offload=cs.HOST)
    check(got, ref, st, pre)
    h2d1, d2h1 = cs.transfer_bytes()
    assert d2h1 - d2h0 == nx * ny * 8            # every output row comes back once
    assert h2d1 - h2d0 >= nx * ny * 8            # every input row goes in at least once


@pytest.mark.parametrize("variant", [cs.XP, cs.XNP, cs.YNP, cs.XYP, cs.XYNP])
def test_host_memory_default_chunks_f32(gpu, variant):
    """Pinned FP32 fields at the default chunk size, DEVICE offload (the output still lands in host
    memory: it is where the field lives)."""
    got, ref, st, pre = run_both(variant, 128, 128, 2, 32, 8, geometry(variant, "sym"), dtype=np.float32, seed=8,
                                 mem="pinned")
    check(got, ref, st, pre)


@pytest.mark.parametrize("variant", [cs.YP, cs.XYP, cs.YNP, cs.XYNP])
def test_swap_sequence(gpu, variant):
    """Create(out=A, in=B); Compute; Swap(A); Compute: the second Compute reads A and writes B, with
    the halo pointers recomputed from the Swap argument (custenCreateDestroy2DYp.cu:235-283)."""
    nx, ny, tiles, bx, by = 64, 96, 3, 16, 8
    H, L, R, V, T, B = geometry(variant, "sym")
    a0 = field(nx, ny, 21)
    w = weights_for(variant, H, V, 4)
    A = sentinel(nx, ny)
    Bf = a0.copy()
    dA, dB, dw = DeviceBuffer.from_array(A), DeviceBuffer.from_array(Bf), DeviceBuffer.from_array(w)
    s = cs.Stencil(variant, nx, ny, dA.ptr, dB.ptr, dw.ptr, H=H, L=L, R=R, V=V, T=T, B=B, num_tiles=tiles,
                   block_x=bx, block_y=by)
    s.compute()
    s.swap(dA.ptr)
    s.compute()
    cs._check(cs.lib().custen_device_synchronize())
    gotA, gotB = dA.download((ny, nx), np.float64), dB.download((ny, nx), np.float64)
    s.destroy()
    refA = A.copy()
    oracle.stencil(variant, refA, Bf, w, num_tiles=tiles, block_x=bx, block_y=by, H=H, L=L, R=R, V=V, T=T, B=B)
    refB = Bf.copy()
    oracle.stencil(variant, refB, refA, w, num_tiles=tiles, block_x=bx, block_y=by, H=H, L=L, R=R, V=V, T=T, B=B)
    assert np.array_equal(gotA, refA)
    assert np.array_equal(gotB, refB)


@pytest.mark.parametrize("variant", [cs.YP, cs.XYP])
def test_swap_with_foreign_halo_source(gpu, variant):
    """Swap(h, C) with C not the new input: the halo rows of every tile come from C, as in the
    reference (the tiles are then not contiguous with their halos and run one launch each)."""
    nx, ny, tiles, bx, by = 64, 64, 2, 16, 8
    H, L, R, V, T, B = geometry(variant, "sym")
    a0, c0 = field(nx, ny, 31), field(nx, ny, 32)
    w = weights_for(variant, H, V, 9)
    A = sentinel(nx, ny)
    dA, dB, dC, dw = (DeviceBuffer.from_array(A), DeviceBuffer.from_array(a0), DeviceBuffer.from_array(c0),
                      DeviceBuffer.from_array(w))
    s = cs.Stencil(variant, nx, ny, dA.ptr, dB.ptr, dw.ptr, H=H, L=L, R=R, V=V, T=T, B=B, num_tiles=tiles,
                   block_x=bx, block_y=by)
    s.swap(dC.ptr)           # now in = A, out = B, halos from C
    dA.upload(a0)
    s.compute()
    cs._check(cs.lib().custen_device_synchronize())
    got = dB.download((ny, nx), np.float64)
    s.destroy()
    ref = a0.copy()
    oracle.stencil(variant, ref, a0, w, num_tiles=tiles, block_x=bx, block_y=by, H=H, L=L, R=R, V=V, T=T, B=B,
                   halo_src=c0)
    assert np.array_equal(got, ref)


def test_weights_reread_every_compute(gpu):
    """Weights are read from memory on every Compute (2d_x_p_kernel.cu:79-83)."""
    nx, ny = 64, 32
    inp = field(nx, ny, 2)
    w1 = np.array([1.0, -2.0, 1.0])
    w2 = np.array([0.5, 0.25, -3.0])
    d_in, d_out, d_w = DeviceBuffer.from_array(inp), DeviceBuffer.from_array(np.zeros_like(inp)), DeviceBuffer.from_array(w1)
    s = cs.Stencil(cs.XP, nx, ny, d_out.ptr, d_in.ptr, d_w.ptr, H=3, L=1, R=1)
    s.compute()
    d_w.upload(w2)
    s.compute()
    cs._check(cs.lib().custen_device_synchronize())
    got = d_out.download((ny, nx), np.float64)
    s.destroy()
    ref = np.zeros_like(inp)
    oracle.stencil(cs.XP, ref, inp, w2, num_tiles=1, block_x=32, block_y=8, H=3, L=1, R=1, V=1, T=0, B=0)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("variant", VARIANTS, ids=cs.VARIANT_NAMES)
@pytest.mark.parametrize("tiles", [1, 2, 4])
@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
def test_parity_tma_path(gpu, variant, tiles, dtype):
    """Geometries the TMA-staged persistent kernel takes (rows tile by 32, columns by 64 / 128 elements,
    16-byte aligned rows): bit-exact, and the TMA kernel is the one that ran."""
    d = 0 if variant < 4 else (1 if variant < 8 else 2)
    fun = variant in (cs.XPFUN, cs.XNPFUN, cs.YPFUN, cs.YNPFUN, cs.XYPFUN, cs.XYNPFUN)
    geom = geometry(variant, "asym" if not fun else "sym")
    fun_id = FUN_IDS[d][1] if fun else -1
    before = cs.kernel_launches_tma()
    got, ref, st, pre = run_both(variant, 256, 128, tiles, 32, 8, geom, dtype=dtype, fun_id=fun_id,
                                 seed=variant + 40 * tiles)
    assert cs.kernel_launches_tma() > before, "the TMA-staged kernel did not run"
    check(got, ref, st, pre)
    assert cs.device_error() == 0


@pytest.mark.parametrize("variant", [cs.XP, cs.YP, cs.XYP, cs.XYNP])
def test_tma_path_periodic_edges_wide_halo(gpu, variant):
    """Halo wider than one 16-byte vector (L = R = T = B = 3): periodic edge tiles take the wrap fix-up."""
    d = 0 if variant < 4 else (1 if variant < 8 else 2)
    geom = {0: (7, 3, 3, 1, 0, 0), 1: (1, 0, 0, 7, 3, 3), 2: (7, 3, 3, 7, 3, 3)}[d]
    before = cs.kernel_launches_tma()
    got, ref, st, pre = run_both(variant, 192, 96, 3, 32, 8, geom, seed=77)
    assert cs.kernel_launches_tma() > before
    check(got, ref, st, pre)


def _wrap_box_cases():
    """(variant, (H, L, R, V, T, B), fun_id): halos on the left only, on the right only, and uneven."""
    cases = []
    for L, R in ((3, 0), (0, 2), (1, 4)):
        cases.append((cs.XP, (L + R + 1, L, R, 1, 0, 0), -1))
        cases.append((cs.XYP, (L + R + 1, L, R, 4, 2, 1), -1))
        cases.append((cs.XYPFUN, (L + R + 1, L, R, 4, 2, 1), FUN_IDS[2][1]))
    cases.append((cs.XPFUN, (5, 2, 2, 1, 0, 0), FUN_IDS[0][1]))   # the 5-point x function
    return cases


@pytest.mark.parametrize("case", _wrap_box_cases(),
                         ids=lambda c: f"{cs.VARIANT_NAMES[c[0]]}-L{c[1][1]}R{c[1][2]}")
@pytest.mark.parametrize("tiles_x", [1, 2])
@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
def test_tma_wrap_boxes(gpu, case, tiles_x, dtype):
    """Wrap-around boxes of the periodic edge columns in the TMA kernel (configuration 0: 64-column FP64
    and 128-column FP32 tiles). With one tile column both boxes land on the same tile; with a halo on one
    side only, one box is issued. Bit-exact, and the TMA kernel is the one that ran."""
    variant, geom, fun_id = case
    nx = (64 if dtype == np.float64 else 128) * tiles_x
    before = cs.kernel_launches_tma()
    got, ref, st, pre = run_both(variant, nx, 64, 1, 16, 8, geom, dtype=dtype, fun_id=fun_id,
                                 seed=nx + geom[1] * 10 + geom[2], config=0)
    assert cs.kernel_launches_tma() > before, "the TMA-staged kernel did not run"
    check(got, ref, st, pre)
    assert cs.device_error() == 0


SHAPES = {  # the compile-time register-window shapes: (variant, H, L, R, V, T, B)
    "X3": (cs.XP, 3, 1, 1, 1, 0, 0), "X5": (cs.XNP, 5, 2, 2, 1, 0, 0), "X9": (cs.XP, 9, 4, 4, 1, 0, 0),
    "Y3": (cs.YNP, 1, 0, 0, 3, 1, 1), "Y5": (cs.YP, 1, 0, 0, 5, 2, 2), "Y9": (cs.YP, 1, 0, 0, 9, 4, 4),
    "XY3": (cs.XYP, 3, 1, 1, 3, 1, 1), "XY5": (cs.XYNP, 5, 2, 2, 5, 2, 2),
}


@pytest.mark.parametrize("shape", list(SHAPES))
@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("dense", [True, False], ids=["dense", "zeros"])
def test_parity_shape_kernels(gpu, shape, dtype, dense):
    """Register sliding-window kernels (compile-time shapes): bit-exact with dense weights and with
    exact-zero weights (FP64 then takes the non-zero list, FP32 keeps every weight in the chain)."""
    v, H, L, R, V, T, B = SHAPES[shape]
    nx, ny, tiles = 256, 128, 2
    inp = field(nx, ny, 7, dtype)
    w = weights_for(v, H, V, 7, dtype, zeros=not dense)
    if dense:
        w[w == 0] = 0.5
    pre = sentinel(nx, ny, dtype)
    ref = pre.copy()
    st = oracle.stencil(v, ref, inp, w, num_tiles=tiles, block_x=32, block_y=8, H=H, L=L, R=R, V=V, T=T, B=B)
    d_in, d_out, d_w = DeviceBuffer.from_array(inp), DeviceBuffer.from_array(pre), DeviceBuffer.from_array(w)
    before = cs.kernel_launches_tma()
    s = cs.Stencil(v, nx, ny, d_out.ptr, d_in.ptr, d_w.ptr, H=H, L=L, R=R, V=V, T=T, B=B, num_tiles=tiles,
                   block_x=32, block_y=8, dtype=cs.F64 if dtype == np.float64 else cs.F32)
    s.compute()
    cs._check(cs.lib().custen_device_synchronize())
    got = d_out.download((ny, nx), dtype)
    s.destroy()
    assert cs.kernel_launches_tma() > before
    check(got, ref, st, pre)


def test_concurrent_handles_from_host_threads(gpu):
    """Independent handles driven from four host threads at once (ctypes releases the GIL during each
    call): the lazily filled per-device tables (device-function addresses, kernel attributes, device
    properties) are shared safely and every result matches the oracle."""
    import threading

    cases = [(cs.XYPFUN, (3, 1, 1, 3, 1, 1), FUN_IDS[2][1]), (cs.XNP, (5, 2, 2, 1, 0, 0), -1),
             (cs.YPFUN, (1, 0, 0, 5, 2, 2), FUN_IDS[1][1]), (cs.XYNP, (5, 2, 2, 5, 2, 2), -1)]
    errors = []

    def worker(k):
        try:
            cs._check(cs.lib().custen_set_device(0))
            variant, geom, fun_id = cases[k]
            d = 0 if variant < 4 else (1 if variant < 8 else 2)
            for rep in range(3):
                got, ref, st, pre = run_both(variant, 128, 64, 2, 32 if d != 1 else 16, 8, geom, fun_id=fun_id,
                                             seed=100 + 10 * k + rep)
                check(got, ref, st, pre)
        except Exception as e:  # reported on the main thread
            errors.append(f"thread {k}: {e!r}")

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errors, errors


def _random_cases(count: int, seed: int):
    """Weighted-stencil geometries drawn within the reference's preconditions: nx % BLOCK_X == 0,
    ny % numTiles == 0, (ny / numTiles) % BLOCK_Y == 0, L, R <= BLOCK_X, T, B <= BLOCK_Y, and at least two
    blocks per direction (the non-periodic and y-periodic kernels assume it)."""
    rng = np.random.default_rng(seed)
    cases = []
    while len(cases) < count:
        variant = int(rng.choice([cs.XP, cs.XNP, cs.YP, cs.YNP, cs.XYP, cs.XYNP]))
        d = 0 if variant < 4 else (1 if variant < 8 else 2)
        bx = int(rng.choice([8, 16, 32]))
        by = int(rng.choice([4, 8, 16]))
        tiles = int(rng.choice([1, 2, 3, 4]))
        nx = bx * int(rng.integers(2, 9))
        ny = by * tiles * int(rng.integers(2, 6))
        L = R = T = B = 0
        if d != 1:
            L, R = int(rng.integers(0, min(4, bx) + 1)), int(rng.integers(0, min(4, bx) + 1))
        if d != 0:
            T, B = int(rng.integers(0, min(4, by) + 1)), int(rng.integers(0, min(4, by) + 1))
        if L + R + T + B == 0:
            continue
        dtype = np.float64 if rng.random() < 0.7 else np.float32
        config = int(rng.integers(0, cs.NUM_CONFIGS)) if rng.random() < 0.5 else None
        cases.append((variant, nx, ny, tiles, bx, by, (L + R + 1, L, R, T + B + 1, T, B), dtype, config))
    return cases


@pytest.mark.parametrize("case", _random_cases(60, 2024), ids=lambda c: f"{cs.VARIANT_NAMES[c[0]]}-{c[1]}x{c[2]}-"
                         f"t{c[3]}-b{c[4]}x{c[5]}-LRTB{c[6][1]}{c[6][2]}{c[6][4]}{c[6][5]}-"
                         f"{'f64' if c[7] == np.float64 else 'f32'}-cfg{c[8]}")
def test_parity_randomized(gpu, case):
    """Random geometries within the reference's preconditions, bit-exact against the oracle on every
    written point, sentinels kept on every untouched one."""
    variant, nx, ny, tiles, bx, by, geom, dtype, config = case
    got, ref, st, pre = run_both(variant, nx, ny, tiles, bx, by, geom, dtype=dtype, seed=nx + ny + tiles,
                                 config=config)
    check(got, ref, st, pre)


@pytest.mark.parametrize("variant", [cs.XYP, cs.YNP])
def test_field_beyond_2gib(gpu, variant):
    """A 16384 x 20480 FP64 field (2.68 GB, element offsets past 2^31 bytes) with small-integer inputs and
    integer weights: every partial sum is exact in FP64, so the result does not depend on summation order
    and plain numpy sums give it bit for bit. Checked on row bands at both ends (periodic wrap across
    them) and around the 2^31-byte offset."""
    import torch
    nx, ny = 16384, 20480
    H, L, R, V, T, B = 5, 2, 2, 5, 2, 2
    if variant == cs.YNP:
        H, L, R = 1, 0, 0
    w = np.random.default_rng(4).integers(-3, 4, H * V).astype(np.float64)
    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev)
    g.manual_seed(7)
    inp = torch.randint(0, 16, (ny, nx), device=dev, generator=g).double()
    out = torch.full((ny, nx), -1.0, device=dev, dtype=torch.float64)
    wt = torch.tensor(w, device=dev)
    s = cs.Stencil(variant, nx, ny, out.data_ptr(), inp.data_ptr(), wt.data_ptr(), H=H, L=L, R=R, V=V, T=T, B=B,
                   block_x=32, block_y=8)
    s.compute()
    torch.cuda.synchronize(dev)
    s.destroy()
    row_2gib = (1 << 31) // (8 * nx)   # first row past the 2^31-byte offset
    bands = [(0, 40), (row_2gib - 20, row_2gib + 20), (ny - 40, ny)]
    for r0, r1 in bands:
        rows = np.arange(r0 - T, r1 + B) % ny
        window = inp[torch.as_tensor(rows, device=dev)].cpu().numpy()
        ref = np.zeros((r1 - r0, nx))
        for j in range(V):
            for i in range(H):
                ref += w[j * H + i] * np.roll(window[j:j + r1 - r0], -(i - L), axis=1)
        got = out[r0:r1].cpu().numpy()
        if variant == cs.YNP:
            # Ynp leaves the field's first T and last B rows untouched (numTiles 1)
            keep = np.ones(r1 - r0, dtype=bool)
            keep[(np.arange(r0, r1) < T) | (np.arange(r0, r1) >= ny - B)] = False
            assert np.all(got[~keep] == -1.0)
            got, ref = got[keep], ref[keep]
        assert np.array_equal(got, ref), f"rows {r0}..{r1}"
    del inp, out
    torch.cuda.empty_cache()
