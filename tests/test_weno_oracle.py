"""The WENO5 advection oracle on the CPU: known answers on smooth fields, and the outputs of the
reference's own kernel (tests/golden/make_golden_weno.py, run on a GB300)."""
from pathlib import Path

import numpy as np
import pytest

import oracle
from custen_gb300.inputs import weno_inputs

GOLDEN = Path(__file__).with_name("golden") / "reference_weno.npz"


@pytest.mark.parametrize("n", [64, 128])
def test_weno_smooth_field_advection_known_answer(n):
    """f = sin(x) cos(2y), constant u = 0.7, v = -1.3: out approximates u df/dx + v df/dy to the
    scheme's high order on a smooth periodic field."""
    h = 2 * np.pi / n
    x = np.arange(n) * h
    f = np.sin(x)[None, :] * np.cos(2 * x)[:, None]
    u = np.full((n, n), 0.7)
    v = np.full((n, n), -1.3)
    exact = 0.7 * np.cos(x)[None, :] * np.cos(2 * x)[:, None] - 1.3 * np.sin(x)[None, :] * (-2) * np.sin(2 * x)[:, None]
    got = oracle.weno(f, u, v, 1.0 / h, 1.0 / h)
    err = np.abs(got - exact).max()
    assert err < (2e-3 if n == 64 else 2e-4), err


def test_weno_convergence_order():
    """Halving h on a smooth field cuts the error by well over 2^3 (fifth order away from the points
    where the smoothness indicators switch stencils)."""
    errs = []
    for n in (32, 64, 128):
        h = 2 * np.pi / n
        x = np.arange(n) * h
        f = np.sin(x)[None, :] + 0.0 * x[:, None]
        u = np.ones((n, n))
        v = np.ones((n, n))
        got = oracle.weno(f, u, v, 1.0 / h, 1.0 / h)
        errs.append(np.abs(got - np.cos(x)[None, :]).max())
    assert errs[0] / errs[1] > 8 and errs[1] / errs[2] > 8, errs


def test_weno_upwind_side_follows_velocity_sign():
    """A step profile advected with u > 0 reads only upwind (left) data: changing values more than two
    points downstream leaves the result unchanged; with u <= 0 the roles swap."""
    n = 32
    f, _, _, dx, dy = weno_inputs(n, n, 1, rough=True)
    u = np.full((n, n), 0.5)
    v = np.zeros((n, n))
    base = oracle.weno(f, u, v, 1 / dx, 1 / dy)
    g = f.copy()
    g[:, 20] += 1.0            # column 20 is 3 points right of column 17
    assert np.array_equal(oracle.weno(g, u, v, 1 / dx, 1 / dy)[:, 17], base[:, 17])
    assert not np.array_equal(oracle.weno(g, -u, v, 1 / dx, 1 / dy)[:, 17], oracle.weno(f, -u, v, 1 / dx, 1 / dy)[:, 17])


# The reference squares its smoothness terms with CUDA's powf, which is not always the correctly rounded
# square the oracle uses: agreement is to the float precision of those terms.
WENO_REL_L2 = 1e-7
WENO_REL_MAX = 1e-7


def weno_close(got, ref):
    rel_l2 = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    rel_max = np.abs(got - ref).max() / np.abs(ref).max()
    return rel_l2 <= WENO_REL_L2 and rel_max <= WENO_REL_MAX, (rel_l2, rel_max)


def test_oracle_reproduces_reference_weno_golden():
    if not GOLDEN.exists():
        pytest.skip("WENO golden fixtures not generated yet")
    g = np.load(GOLDEN)
    assert len(g["configs"]) == 5
    for i, cfg in enumerate(g["configs"]):
        nx, ny, tiles, bx, by, rough = (int(c) for c in cfg)
        f, u, v, dx, dy = weno_inputs(nx, ny, 200 + i, rough=bool(rough))
        got = oracle.weno(f, u, v, 1.0 / dx, 1.0 / dy)
        ok, err = weno_close(got, g[f"out_{i}"])
        assert ok, f"config {i} {cfg.tolist()}: rel L2 {err[0]:.2e}, rel max {err[1]:.2e}"
