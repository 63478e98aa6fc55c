"""The CPU oracle against golden outputs of the reference's own kernels (tests/golden/make_golden.py,
run on a GB300 with the reference kernels compiled unchanged from the reference sources)."""
from pathlib import Path

import numpy as np
import pytest

import oracle
from custen_gb300.inputs import field, sentinel
from tests.helpers import weights_for

GOLDEN = Path(__file__).with_name("golden") / "reference_kernels.npz"


@pytest.fixture(scope="module")
def golden():
    if not GOLDEN.exists():
        pytest.skip("golden fixtures not generated yet")
    return np.load(GOLDEN)


def test_oracle_reproduces_reference_golden_outputs(golden):
    cfgs = golden["configs"]
    assert len(cfgs) == 24
    for i, cfg in enumerate(cfgs):
        v, nx, ny, tiles, bx, by, H, L, R, V, T, B, fun_id = (int(c) for c in cfg)
        seed = 100 + i
        inp = field(nx, ny, seed)
        if fun_id >= 0:
            ncoef = {0: 1, 1: 5, 2: 9, 3: 5, 4: H * V, 5: H * V}[fun_id]
            coef = np.random.default_rng(50 + seed).uniform(-1, 1, ncoef)
        else:
            coef = weights_for(v, H, V, seed)
        pre = sentinel(nx, ny)
        ora = pre.copy()
        st = oracle.stencil(v, ora, inp, coef, num_tiles=tiles, block_x=bx, block_y=by, H=H, L=L, R=R, V=V, T=T,
                            B=B, fun_id=fun_id)
        ref = golden[f"out_{i}"]
        written = st == 1
        if v == 5:  # kernel2DYnp: last block row of the last tile has no barrier (2d_y_np_kernel.cu:227-249)
            written[ny - by:, :] = False
        assert np.array_equal(ref[written], ora[written]), f"config {i} {cfg.tolist()}: written points differ"
        assert np.array_equal(ref[st == 0], pre[st == 0]), f"config {i}: untouched points differ"
