"""The stencil oracle against the known answers of the reference examples (examples/src/*.cu).

The reference ships no test suite; its examples print each result beside an analytic answer. These
tests run the same fields, stencils and tilings (shrunk where the example grid is large) through the
CPU oracle and check the analytic answers within the finite-difference truncation error, plus the
points each example leaves untouched or zeroed.
"""
import math

import numpy as np
import pytest

import custen_gb300 as cs
import oracle

W9 = np.array([-1 / 560, 8 / 315, -1 / 5, 8 / 5, -205 / 72, 8 / 5, -1 / 5, 8 / 315, -1 / 560])  # examples/src/2d_x_p.cu:99-114
W3 = np.array([1.0, -2.0, 1.0])                                                              # examples/src/2d_y_p.cu:106-108
WXY = np.array([1.0, 0.0, -1.0, 0.0, 0.0, 0.0, -1.0, 0.0, 1.0])                               # examples/src/2d_xy_p.cu:110-120


def run(variant, inp, coef, **kw):
    out = np.zeros_like(inp)
    st = oracle.stencil(variant, out, inp, coef, **kw)
    return out, st


def test_x_periodic_9pt():  # examples/src/2d_x_p.cu: 2048x1024, 2 tiles, 32x32 (shrunk)
    nx, ny = 512, 64
    dx = 2 * math.pi / nx
    x = np.arange(nx) * dx
    inp = np.tile(np.sin(x), (ny, 1))
    out, st = run(cs.XP, inp, W9 / dx**2, num_tiles=2, block_x=32, block_y=32, H=9, L=4, R=4, V=1, T=0, B=0)
    assert (st == 1).all()
    np.testing.assert_allclose(out, -inp, atol=1e-9)


def test_x_nonperiodic_9pt():  # examples/src/2d_x_np.cu: 1024x512, dx = 2pi/(nx-1)
    nx, ny = 256, 32
    dx = 2 * math.pi / (nx - 1)
    x = np.arange(nx) * dx
    inp = np.tile(np.sin(x), (ny, 1))
    out, st = run(cs.XNP, inp, W9 / dx**2, num_tiles=1, block_x=32, block_y=16, H=9, L=4, R=4, V=1, T=0, B=0)
    assert (st[:, :4] == 0).all() and (out[:, :4] == 0).all()          # left edge untouched
    assert (st[:, -4:] == 1).all() and (out[:, -4:] == 0.0).all()       # right edge written as 0.0
    np.testing.assert_allclose(out[:, 4:-4], -inp[:, 4:-4], atol=1e-7)


def test_y_periodic_3pt():  # examples/src/2d_y_p.cu: 512^2, 1 tile, 8x8, 3-point
    nx, ny = 64, 512
    dy = 2 * math.pi / ny
    y = np.arange(ny) * dy
    inp = np.tile(np.sin(y)[:, None], (1, nx))
    out, st = run(cs.YP, inp, W3 / dy**2, num_tiles=1, block_x=8, block_y=8, H=1, L=0, R=0, V=3, T=1, B=1)
    assert (st == 1).all()
    np.testing.assert_allclose(out, -inp, atol=5e-5)


@pytest.mark.parametrize("tiles", [1, 2, 4])
def test_y_nonperiodic_9pt(tiles):  # examples/src/2d_y_np.cu: 512^2, 2 tiles, 8x8
    nx, ny = 32, 256
    dy = 2 * math.pi / (ny - 1)
    y = np.arange(ny) * dy
    inp = np.tile(np.sin(y)[:, None], (1, nx))
    out, st = run(cs.YNP, inp, W9 / dy**2, num_tiles=tiles, block_x=8, block_y=8, H=1, L=0, R=0, V=9, T=4, B=4)
    assert (st[:4] == 0).all() and (st[-4:] == 0).all()
    assert (st[4:-4] == 1).all()
    np.testing.assert_allclose(out[4:-4], -inp[4:-4], atol=1e-7)


@pytest.mark.parametrize("tiles", [1, 2])
def test_xy_periodic_cross(tiles):  # examples/src/2d_xy_p.cu: 8192^2, 1 tile, 32x32 (shrunk)
    nx, ny = 256, 128
    dx, dy = 2 * math.pi / nx, 2 * math.pi / ny
    x, y = np.arange(nx) * dx, np.arange(ny) * dy
    inp = np.sin(x)[None, :] * np.cos(y)[:, None]
    out, st = run(cs.XYP, inp, WXY / (4 * dx * dy), num_tiles=tiles, block_x=32, block_y=32, H=3, L=1, R=1, V=3,
                  T=1, B=1)
    assert (st == 1).all()
    np.testing.assert_allclose(out, -np.cos(x)[None, :] * np.sin(y)[:, None], atol=2e-3)


def test_xy_nonperiodic_cross_4tiles():  # examples/src/2d_xy_np.cu: 128^2, 4 tiles, 4x4 blocks
    nx = ny = 128
    dx = dy = 2 * math.pi / (nx - 1)
    x, y = np.arange(nx) * dx, np.arange(ny) * dy
    inp = np.sin(x)[None, :] * np.cos(y)[:, None]
    out, st = run(cs.XYNP, inp, WXY / (4 * dx * dy), num_tiles=4, block_x=4, block_y=4, H=3, L=1, R=1, V=3,
                  T=1, B=1)
    ans = -np.cos(x)[None, :] * np.sin(y)[:, None]
    assert (st[0, :] == 0).all() and (st[-1, :] == 0).all() and (st[:, 0] == 0).all() and (st[:, -1] == 0).all()
    assert (st[1:-1, 1:-1] == 1).all()
    np.testing.assert_allclose(out[1:-1, 1:-1], ans[1:-1, 1:-1], atol=2e-2)


def test_x_nonperiodic_fun():  # examples/src/2d_x_np_fun.cu: f = (d[-1] - 2 d[0] + d[1]) * coe[0]
    nx, ny = 256, 64
    dx = 2 * math.pi / (nx - 1)
    x = np.arange(nx) * dx
    inp = np.tile(np.sin(x), (ny, 1))
    coe = np.array([1.0 / dx**2])
    out, st = run(cs.XNPFUN, inp, coe, num_tiles=4, block_x=32, block_y=16, H=3, L=1, R=1, V=1, T=0, B=0,
                  fun_id=0)
    assert (st[:, 0] == 0).all() and (st[:, -1] == 0).all() and (st[:, 1:-1] == 1).all()
    np.testing.assert_allclose(out[:, 1:-1], -inp[:, 1:-1], atol=1e-3)


@pytest.mark.parametrize("variant", [cs.YPFUN, cs.YNPFUN])
def test_y_fun_9pt(variant):  # examples/src/2d_y_p_fun.cu (64^2, 4 tiles, 4x4) and 2d_y_np_fun.cu
    nx, ny = 16, 64
    periodic = variant == cs.YPFUN
    dy = 2 * math.pi / (ny if periodic else ny - 1)
    y = np.arange(ny) * dy
    inp = np.tile(np.sin(y)[:, None], (1, nx))
    out, st = run(variant, inp, W9 / dy**2, num_tiles=4, block_x=4, block_y=4, H=1, L=0, R=0, V=9, T=4, B=4,
                  fun_id=2)
    sl = slice(None) if periodic else slice(4, -4)
    assert (st[sl] == 1).all()
    np.testing.assert_allclose(out[sl], -inp[sl], atol=1e-6)


@pytest.mark.parametrize("variant", [cs.XYPFUN, cs.XYNPFUN])
def test_xy_fun_cross(variant):  # examples/src/2d_xy_p_fun.cu (16x32 blocks) and 2d_xy_np_fun.cu (8x8)
    nx = ny = 128
    periodic = variant == cs.XYPFUN
    dx = dy = 2 * math.pi / (nx if periodic else nx - 1)
    x, y = np.arange(nx) * dx, np.arange(ny) * dy
    inp = np.sin(x)[None, :] * np.cos(y)[:, None]
    bx, by = (16, 32) if periodic else (8, 8)
    out, st = run(variant, inp, WXY / (4 * dx * dy), num_tiles=1, block_x=bx, block_y=by, H=3, L=1, R=1, V=3, T=1,
                  B=1, fun_id=4)
    ans = -np.cos(x)[None, :] * np.sin(y)[:, None]
    sl = (slice(None), slice(None)) if periodic else (slice(1, -1), slice(1, -1))
    assert (st[sl] == 1).all()
    np.testing.assert_allclose(out[sl], ans[sl], atol=2e-2)


def test_xyp_matches_plain_host_loop():
    """The block emulation of kernel2DXYp equals a plain modular-index loop (same FMA order)."""
    rng = np.random.default_rng(7)
    nx, ny = 96, 64
    inp = rng.standard_normal((ny, nx))
    w = rng.standard_normal(25)
    out, st = run(cs.XYP, inp, w, num_tiles=2, block_x=32, block_y=8, H=5, L=2, R=2, V=5, T=2, B=2)
    ref = oracle.host_loop_xyp(inp, w, 5, 2, 5, 2)
    assert (st == 1).all()
    assert np.array_equal(out, ref)


def test_xynp_right_edge_guard_quirk():
    """kernel2DXYnp guards the right-edge middle blocks with BX - L (2d_xy_np_kernel.cu:862):
    with L > R the points x in [nx-L, nx-R) of middle block rows are left untouched; with L < R the
    reference reads shared memory it never loaded there (status 2)."""
    rng = np.random.default_rng(3)
    nx, ny = 64, 48
    inp = rng.standard_normal((ny, nx))
    w = rng.standard_normal(4 * 3)
    out, st = run(cs.XYNP, inp, w, num_tiles=1, block_x=16, block_y=8, H=4, L=2, R=1, V=3, T=1, B=1)
    mid = slice(8, 40)  # block rows 1..4 (not the first/last)
    assert (st[mid, nx - 2] == 0).all() and (st[mid, nx - 3] == 1).all()
    out2, st2 = run(cs.XYNP, inp, w, num_tiles=1, block_x=16, block_y=8, H=4, L=1, R=2, V=3, T=1, B=1)
    assert (st2[mid, nx - 2] == 2).all()
