"""Parity of the persistent TMA stencil kernel when every CTA walks many tiles (GPU).

The TMA-staged kernel is persistent: CTA b takes tiles b, b + grid, b + 2 grid, ... through a ring of S = 3
shared-memory stages, re-filling a stage (new mbarrier phase, new window box and, on the first and last tile
column of a periodic launch, new wrap-around boxes) as soon as its tile is done. On the small fields of the
other parity tests the grid covers every tile at once, so no stage is ever reused. Here
custen_set_max_ctas caps the grid at two CTAs, so each CTA takes nine tiles (three rounds of the ring, with
first, middle and last tile columns landing in recycled stages), in every tile configuration, for the twelve
operators of the plain stencil sweep in FP64 and FP32, the c^3 - c Fun operators both fused and through the
indirect call. Every written point must be bit-identical to the oracle and every untouched point must keep
its sentinel.

The last tests run the benchmark's own operators (4th-order d2/dx2, cross derivative, c^3 - c Laplacian) on
its own field sin(3x)cos(5y) + U(-1e-3, 1e-3) at 2048^2 with the uncapped grid -- 2048 tiles for 456 CTAs --
and compare the library bit for bit with the oracle and with the reference's own kernels rebuilt for sm_103a.
"""
import numpy as np
import pytest

import custen_gb300 as cs
import oracle
from custen_gb300.buffers import DeviceBuffer
from custen_gb300.inputs import field, sentinel, sweep_operators
from tests.test_stencil_parity import check, run_both

pytestmark = pytest.mark.gpu

TILES_X, TILES_Y, CAP = 3, 6, 2          # 18 tiles, 9 per CTA: every stage is used three times
F64_TILES = [(64, 32), (32, 32), (64, 16), (64, 32), (64, 64), (32, 16)]    # stencil_configs.h, per entry
F32_TILES = [(128, 32), (64, 32), (128, 16), (128, 32), (128, 64), (64, 16)]
FUN = (cs.XPFUN, cs.XNPFUN, cs.YPFUN, cs.YNPFUN, cs.XYPFUN, cs.XYNPFUN)


@pytest.fixture
def capped_grid():
    cs.set_max_ctas(CAP)
    yield
    cs.set_max_ctas(0)


def sweep_case(variant, n):
    """(H, L, R, V, T, B), coefficients and fun_id of the sweep operator `variant`, scaled for an n-grid."""
    for _, v, H, L, R, V, T, B, w, fun_id, _ in sweep_operators(n):
        if v == variant:
            return (H, L, R, V, T, B), np.array(w), fun_id
    raise KeyError(variant)


def run_capped(variant, dtype, cfg, tiles, seed):
    tw, th = (F64_TILES if dtype == np.float64 else F32_TILES)[cfg]
    nx, ny = TILES_X * tw, TILES_Y * th
    geom, w, fun_id = sweep_case(variant, nx)
    before = cs.kernel_launches_tma()
    got, ref, st, pre = run_sweep_operator(variant, nx, ny, tiles, 32, 8, geom, w, fun_id, dtype, seed, cfg)
    assert cs.kernel_launches_tma() > before, "the TMA-staged kernel did not run"
    return got, ref, st, pre


def run_sweep_operator(variant, nx, ny, tiles, bx, by, geom, w, fun_id, dtype, seed, cfg=None):
    """One operator of the sweep through the library with the sweep's own coefficients; the oracle beside it."""
    H, L, R, V, T, B = geom
    inp = field(nx, ny, seed, dtype)
    coef = np.asarray(w, dtype=dtype)
    pre = sentinel(nx, ny, dtype)
    ref = pre.copy()
    st = oracle.stencil(variant, ref, inp, coef, num_tiles=tiles, block_x=bx, block_y=by, H=H, L=L, R=R, V=V, T=T,
                        B=B, fun_id=fun_id)
    dt = cs.F64 if dtype == np.float64 else cs.F32
    d_in, d_out, d_c = DeviceBuffer.from_array(inp), DeviceBuffer.from_array(pre), DeviceBuffer.from_array(coef)
    func = cs.builtin_function(fun_id, dt) if fun_id >= 0 else None
    s = cs.Stencil(variant, nx, ny, d_out.ptr, d_in.ptr, d_c.ptr, H=H, L=L, R=R, V=V, T=T, B=B, num_tiles=tiles,
                   block_x=bx, block_y=by, dtype=dt, ncoef=coef.size, func=func)
    if cfg is not None:
        s.set_config(cfg)
    s.compute()
    cs._check(cs.lib().custen_device_synchronize())
    got = d_out.download((ny, nx), dtype)
    s.destroy()
    return got, ref, st, pre


@pytest.mark.parametrize("variant", list(range(12)), ids=cs.VARIANT_NAMES)
@pytest.mark.parametrize("cfg", list(range(cs.NUM_CONFIGS)))
@pytest.mark.parametrize("tiles", [1, 4])
@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
def test_ring_reuse_sweep_operators(gpu, capped_grid, variant, cfg, tiles, dtype):
    """The sweep's operators with the grid capped at two CTAs, every tile configuration, numTiles 1 and 4:
    bit-exact, sentinels kept, no device error (the Fun operators run fused here)."""
    got, ref, st, pre = run_capped(variant, dtype, cfg, tiles, seed=100 + 7 * variant + cfg)
    check(got, ref, st, pre)
    assert cs.device_error() == 0


@pytest.mark.parametrize("variant", FUN, ids=[cs.VARIANT_NAMES[v] for v in FUN])
@pytest.mark.parametrize("cfg", list(range(cs.NUM_CONFIGS)))
@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
def test_ring_reuse_indirect_fun(gpu, capped_grid, variant, cfg, dtype):
    """The same c^3 - c Fun operators through the indirect device-function call (fusion off), capped grid:
    bit-exact, and bitwise equal to the fused path."""
    got_fused, ref, st, pre = run_capped(variant, dtype, cfg, 2, seed=300 + variant + cfg)
    cs.set_fun_fusion(False)
    try:
        got_call, *_ = run_capped(variant, dtype, cfg, 2, seed=300 + variant + cfg)
    finally:
        cs.set_fun_fusion(True)
    check(got_call, ref, st, pre)
    assert got_fused.tobytes() == got_call.tobytes()
    assert cs.device_error() == 0


def _wrap_cases():
    """Uneven periodic halos: one wrap-around box or two of different widths, re-issued into recycled stages."""
    return [(cs.XP, (5, 3, 1, 1, 0, 0)), (cs.XP, (3, 0, 2, 1, 0, 0)), (cs.XYP, (4, 2, 1, 3, 1, 1)),
            (cs.XYP, (6, 1, 4, 4, 2, 1)), (cs.XNP, (5, 3, 1, 1, 0, 0)), (cs.XYNP, (4, 2, 1, 3, 1, 1))]


@pytest.mark.parametrize("case", _wrap_cases(), ids=lambda c: f"{cs.VARIANT_NAMES[c[0]]}-L{c[1][1]}R{c[1][2]}")
@pytest.mark.parametrize("cfg", [0, 1, 4, 5])
@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
def test_ring_reuse_uneven_halos(gpu, capped_grid, case, cfg, dtype):
    """Asymmetric halos with random weights (exact zeros included) on the capped grid: bit-exact."""
    variant, geom = case
    tw, th = (F64_TILES if dtype == np.float64 else F32_TILES)[cfg]
    got, ref, st, pre = run_both(variant, TILES_X * tw, TILES_Y * th, 2, 32, 8, geom, dtype=dtype,
                                 seed=500 + variant + cfg, config=cfg)
    check(got, ref, st, pre)
    assert cs.device_error() == 0


N_BENCH = 2048


@pytest.mark.parametrize("variant", list(range(12)), ids=cs.VARIANT_NAMES)
@pytest.mark.parametrize("tiles", [1, 4])
def test_sweep_operators_2048_bit_exact_vs_oracle(gpu, variant, tiles):
    """The sweep at 2048^2 (FP64, the benchmark's field, default tile configuration, uncapped grid: about
    4.5 tiles per CTA): bit-exact against the oracle on every written point."""
    geom, w, fun_id = sweep_case(variant, N_BENCH)
    got, ref, st, pre = run_sweep_operator(variant, N_BENCH, N_BENCH, tiles, 32, 8, geom, w, fun_id, np.float64,
                                           seed=1, cfg=0)
    check(got, ref, st, pre)
    assert cs.device_error() == 0


@pytest.fixture(scope="module")
def ref_kernels(gpu):
    R = oracle.reference_kernels()
    if R is None:
        pytest.skip("reference kernel cubin (oracle/_ref) not present: build it where the reference sources are")
    return R


@pytest.mark.parametrize("variant", list(range(12)), ids=cs.VARIANT_NAMES)
@pytest.mark.parametrize("tiles", [1, 4])
@pytest.mark.parametrize("block", [(32, 8), (32, 32)], ids=["32x8", "32x32"])
def test_sweep_operators_2048_bit_exact_vs_reference_kernels(ref_kernels, variant, tiles, block):
    """The sweep at 2048^2 through the library (autotuned tile configuration) and through the reference's own
    kernels (rebuilt for sm_103a, reference tile loop) on the same device buffers: identical on every point
    the reference writes deterministically; the points it leaves untouched keep the sentinel in both."""
    bx, by = block
    geom, w, fun_id = sweep_case(variant, N_BENCH)
    H, L, R, V, T, B = geom
    n = N_BENCH
    inp = field(n, n, 1)
    pre = sentinel(n, n)
    d_in, d_w = DeviceBuffer.from_array(inp), DeviceBuffer.from_array(np.asarray(w))
    d_ref, d_lib = DeviceBuffer.from_array(pre), DeviceBuffer.from_array(pre)
    d = 0 if variant < 4 else (1 if variant < 8 else 2)
    num_sten = H * V if d == 2 else (H if d == 0 else V)
    oracle.reference_compute(variant, n, n, tiles, bx, by, d_ref.ptr, d_in.ptr, d_w.ptr, num_sten=num_sten, H=H,
                             L=L, R=R, V=V, T=T, B=B, num_coe=len(w),
                             func=oracle.reference_fun_ptr(fun_id) if fun_id >= 0 else 0)
    s = cs.Stencil(variant, n, n, d_lib.ptr, d_in.ptr, d_w.ptr, H=H, L=L, R=R, V=V, T=T, B=B, num_tiles=tiles,
                   block_x=bx, block_y=by, ncoef=len(w), func=cs.builtin_function(fun_id) if fun_id >= 0 else None)
    s.autotune()
    s.compute()
    cs._check(cs.lib().custen_device_synchronize())
    got_ref = d_ref.download((n, n), np.float64)
    got_lib = d_lib.download((n, n), np.float64)
    s.destroy()
    st = oracle.stencil(variant, pre.copy(), inp, np.asarray(w), num_tiles=tiles, block_x=bx, block_y=by, H=H, L=L,
                        R=R, V=V, T=T, B=B, fun_id=fun_id)
    written = st == 1
    if variant == cs.YNP:   # the reference's last block row has no barrier (2d_y_np_kernel.cu:227-249)
        written[n - by:] = False
    assert np.array_equal(got_lib[written], got_ref[written]), (
        f"library differs from the reference kernel at {int((got_lib[written] != got_ref[written]).sum())} points")
    untouched = st == 0
    assert np.array_equal(got_ref[untouched], pre[untouched])
    assert np.array_equal(got_lib[untouched], pre[untouched])
    assert cs.device_error() == 0
