"""The batched pentadiagonal oracle on the CPU: solutions satisfy the systems, and the factors and
solutions equal those of the reference's own kernels (tests/golden/make_golden_pent.py, on a GB300)."""
from pathlib import Path

import numpy as np
import pytest

import oracle
from custen_gb300.inputs import pent_system
from tests.helpers import pent_dense_apply

GOLDEN = Path(__file__).with_name("golden") / "reference_pent.npz"


@pytest.mark.parametrize("m,batch", [(4, 3), (5, 7), (40, 16), (257, 9)])
def test_pent_oracle_solves_the_systems(m, batch):
    ds, dl, d, du, dw, b = pent_system(m, batch, 1)
    f = oracle.pent_factor(ds, dl, d, du, dw)
    x = oracle.pent_solve(f, b)
    r = pent_dense_apply(ds, dl, d, du, dw, x) - b
    assert np.abs(r).max() < 1e-13


def test_pent_oracle_reproduces_reference_kernels():
    if not GOLDEN.exists():
        pytest.skip("pentadiagonal golden fixtures not generated yet")
    g = np.load(GOLDEN)
    for k, (m, batch) in enumerate(g["configs"]):
        m, batch = int(m), int(batch)
        ds, dl, d, du, dw, b = pent_system(m, batch, k)
        f = oracle.pent_factor(ds, dl, d, du, dw)
        for name, arr in zip(("ds", "dl", "d", "du", "dw"), f):
            assert np.array_equal(arr, g[f"{name}_{k}"]), (k, name)
        assert np.array_equal(oracle.pent_solve(f, b), g[f"x_{k}"]), k
