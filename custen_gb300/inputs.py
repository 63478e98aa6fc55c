"""Seeded synthetic inputs of the benchmark workloads.

field(): sin(3x)cos(5y) + U(-1e-3, 1e-3) on a periodic [0, 2 pi)^2 grid, the plain stencil sweep's input.
sentinel(): a recognisable pre-fill of an output field (cells an operator leaves untouched keep it).
weno_inputs(): advected field and velocities of the WENO5 advection operator.
pent_system(): diagonally dominant batched pentadiagonal systems in cuPentBatch's interleaved layout.
sweep_operators(): the twelve operators of the plain stencil sweep (weights, windows, Fun functions).
"""
from __future__ import annotations

import math

import numpy as np

# 4th-order d2/dx2, the 3x3 cross derivative and the 5-point Laplacian (unscaled)
W5 = [-1.0, 16.0, -30.0, 16.0, -1.0]
WCROSS = [1.0, 0.0, -1.0, 0.0, 0.0, 0.0, -1.0, 0.0, 1.0]
WLAP = [0.0, 1.0, 0.0, 1.0, -4.0, 1.0, 0.0, 1.0, 0.0]


def sweep_operators(n: int):
    """The plain stencil sweep on an n x n periodic grid, h = 2 pi / n: X and Y 5-point 4th-order d2/dx2
    weights [-1, 16, -30, 16, -1] / (12 h^2), the XY 3 x 3 cross derivative [1, 0, -1; 0, 0, 0; -1, 0, 1] /
    (4 h^2), and Fun variants applying c^3 - c before the weights (X / Y: the same 5-point weights through
    shipped function ids 1 / 3; XY: the 5-point Laplacian [0, 1, 0; 1, -4, 1; 0, 1, 0] / h^2 through id 5,
    the Cahn-Hilliard nonLinRHS form).

    Returns (name, variant, H, L, R, V, T, B, weights, fun_id, fp64_ops_per_point) per operator; fun_id is
    -1 for the weighted variants. The FP64 operation count skips exact-zero weights, and for the Fun
    variants counts c^3 - c once per input value (the fused form) plus one FMA per non-zero coefficient."""
    h = 2 * math.pi / n
    w5 = [w / (12 * h * h) for w in W5]
    wc = [w / (4 * h * h) for w in WCROSS]
    wl = [w / (h * h) for w in WLAP]
    ops = []
    for nm, v in (("Xp", 0), ("Xnp", 1)):
        ops.append((nm, v, 5, 2, 2, 1, 0, 0, w5, -1, 5))
    for nm, v in (("XpFun", 2), ("XnpFun", 3)):
        ops.append((nm, v, 5, 2, 2, 1, 0, 0, w5, 1, 7))
    for nm, v in (("Yp", 4), ("Ynp", 5)):
        ops.append((nm, v, 1, 0, 0, 5, 2, 2, w5, -1, 5))
    for nm, v in (("YpFun", 6), ("YnpFun", 7)):
        ops.append((nm, v, 1, 0, 0, 5, 2, 2, w5, 3, 7))
    for nm, v in (("XYp", 8), ("XYnp", 9)):
        ops.append((nm, v, 3, 1, 1, 3, 1, 1, wc, -1, 4))
    for nm, v in (("XYpFun", 10), ("XYnpFun", 11)):
        ops.append((nm, v, 3, 1, 1, 3, 1, 1, wl, 5, 7))
    return ops


def field(nx: int, ny: int, seed: int, dtype=np.float64) -> np.ndarray:
    """sin(3x)cos(5y) + U(-1e-3, 1e-3) on [0,2pi)^2 (the benchmark field)."""
    rng = np.random.default_rng(seed)
    x = np.arange(nx) * (2 * np.pi / nx)
    y = np.arange(ny) * (2 * np.pi / ny)
    f = np.sin(3 * x)[None, :] * np.cos(5 * y)[:, None] + rng.uniform(-1e-3, 1e-3, size=(ny, nx))
    return np.ascontiguousarray(f.astype(dtype))


def sentinel(nx: int, ny: int, dtype=np.float64) -> np.ndarray:
    """Pre-fill of the output: distinct, finite, recognisable values."""
    return (np.arange(nx * ny, dtype=np.float64).reshape(ny, nx) * 1e-3 + 12345.0).astype(dtype)


def weno_inputs(nx: int, ny: int, seed: int, rough: bool = False):
    """Advected field, velocities and spacings for the WENO operator: the benchmark field (or, rough,
    a random one that drives the nonlinear weights), u and v of both signs with some exact zeros (the
    reference's `> 0.0` test sends them to the other upwind side), dx = 2 pi / nx, dy = 2 pi / ny."""
    rng = np.random.default_rng(500 + seed)
    f = rng.standard_normal((ny, nx)) if rough else field(nx, ny, seed)
    u = rng.uniform(-1.0, 1.0, (ny, nx))
    v = rng.uniform(-1.0, 1.0, (ny, nx))
    u[rng.random((ny, nx)) < 0.05] = 0.0
    v[rng.random((ny, nx)) < 0.05] = 0.0
    return (np.ascontiguousarray(f), np.ascontiguousarray(u), np.ascontiguousarray(v), 2 * np.pi / nx,
            2 * np.pi / ny)


def pent_system(m: int, batch: int, seed: int):
    """Diagonally dominant batched pentadiagonal systems in the interleaved layout (arrays of shape
    (m, batch), element [i, s] = row i of system s): ds, dl, d, du, dw and a right-hand side b, with the
    zero entries of cuPentBatch's convention (ds rows 0-1, dl row 0, du row m-1, dw rows m-2, m-1)."""
    rng = np.random.default_rng(900 + seed)
    ds, dl, du, dw = (rng.uniform(-1.0, 1.0, (m, batch)) for _ in range(4))
    d = rng.uniform(5.0, 8.0, (m, batch)) * np.where(rng.random((m, batch)) < 0.5, 1.0, -1.0)
    ds[:2] = 0.0
    dl[:1] = 0.0
    du[m - 1:] = 0.0
    dw[m - 2:] = 0.0
    b = rng.uniform(-1.0, 1.0, (m, batch))
    return [np.ascontiguousarray(a) for a in (ds, dl, d, du, dw, b)]
