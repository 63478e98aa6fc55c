"""Pins the oracle, and this library, to the reference's own kernels (GPU).

The reference cuSten kernels are compiled unchanged from the reference sources for sm_103a
(oracle/ref_build.py) and launched with the reference's tile loop (oracle/ref_runner.cpp). On the same
inputs, the oracle must reproduce every point the reference writes deterministically, bit for bit,
and leave the same points untouched; the library must match both.

Known non-determinism of the reference, excluded from the bit comparison and reported instead:
  - kernel2DYnp's last block row of the last tile reads shared memory without a barrier
    (2d_y_np_kernel.cu:227-249);
  - kernel2DXYnp(Fun) writes, for L < R, right-edge middle-block points computed from shared memory
    it never loaded (oracle status 2).
"""
import numpy as np
import pytest

import custen_gb300 as cs
import oracle
from custen_gb300.buffers import DeviceBuffer
from custen_gb300.inputs import field, sentinel
from tests.helpers import weights_for
from tests.test_stencil_parity import FUN_IDS, geometry

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref(gpu):
    R = oracle.reference_kernels()
    if R is None:
        pytest.skip("reference kernel cubin (oracle/_ref) not present: build it where the reference sources are")
    return R


def run_reference_and_oracle(variant, nx, ny, tiles, bx, by, geom, fun_id=-1, seed=0):
    H, L, R, V, T, B = geom
    inp = field(nx, ny, seed)
    fun = fun_id >= 0
    if fun:
        ncoef = {0: 1, 1: 5, 2: 9, 3: 5, 4: H * V, 5: H * V}[fun_id]
        coef = np.random.default_rng(50 + seed).uniform(-1, 1, ncoef)
    else:
        coef = weights_for(variant, H, V, seed)
        ncoef = coef.size
    pre = sentinel(nx, ny)
    d_in, d_out, d_c = DeviceBuffer.from_array(inp), DeviceBuffer.from_array(pre), DeviceBuffer.from_array(coef)
    d = 0 if variant < 4 else (1 if variant < 8 else 2)
    num_sten = H * V if d == 2 else (H if d == 0 else V)
    oracle.reference_compute(variant, nx, ny, tiles, bx, by, d_out.ptr, d_in.ptr, d_c.ptr, num_sten=num_sten, H=H,
                             L=L, R=R, V=V, T=T, B=B, num_coe=ncoef,
                             func=oracle.reference_fun_ptr(fun_id) if fun else 0)
    got_ref = d_out.download((ny, nx), np.float64)
    ora = pre.copy()
    st = oracle.stencil(variant, ora, inp, coef, num_tiles=tiles, block_x=bx, block_y=by, H=H, L=L, R=R, V=V,
                        T=T, B=B, fun_id=fun_id)
    # the library on the same inputs
    d_out2 = DeviceBuffer.from_array(pre)
    s = cs.Stencil(variant, nx, ny, d_out2.ptr, d_in.ptr, d_c.ptr, H=H, L=L, R=R, V=V, T=T, B=B, num_tiles=tiles,
                   block_x=bx, block_y=by, ncoef=ncoef, func=cs.builtin_function(fun_id) if fun else None)
    s.compute()
    cs._check(cs.lib().custen_device_synchronize())
    got_lib = d_out2.download((ny, nx), np.float64)
    s.destroy()
    return got_ref, ora, got_lib, st, pre


def racy_rows(variant, ny, tiles, by):
    if variant != cs.YNP:
        return np.zeros(ny, dtype=bool)
    r = np.zeros(ny, dtype=bool)
    r[ny - by:] = True
    return r


@pytest.mark.parametrize("variant", list(range(12)), ids=cs.VARIANT_NAMES)
@pytest.mark.parametrize("tiles", [1, 2, 4])
@pytest.mark.parametrize("kind", ["sym", "asym"])
def test_oracle_and_library_match_reference_kernels(ref, variant, tiles, kind):
    d = 0 if variant < 4 else (1 if variant < 8 else 2)
    geom = geometry(variant, kind)
    fun = variant in (cs.XPFUN, cs.XNPFUN, cs.YPFUN, cs.YNPFUN, cs.XYPFUN, cs.XYNPFUN)
    fun_id = -1
    if fun:
        fun_id = FUN_IDS[d][1]
        if d == 1:
            geom = (1, 0, 0, 5, 2, 2)
        elif d == 0:
            geom = (5, 2, 2, 1, 0, 0)
    nx, ny = (96, 64) if d != 1 else (48, 128)
    bx, by = (32 if d != 1 else 16), 8
    got_ref, ora, got_lib, st, pre = run_reference_and_oracle(variant, nx, ny, tiles, bx, by, geom, fun_id,
                                                              seed=variant * 7 + tiles)
    racy = racy_rows(variant, ny, tiles, by)[:, None] & np.ones((1, nx), dtype=bool)
    written = (st == 1) & ~racy
    assert np.array_equal(got_ref[written], ora[written]), (
        f"oracle differs from the reference kernel at {int((got_ref[written] != ora[written]).sum())} points")
    untouched = st == 0
    assert np.array_equal(got_ref[untouched], pre[untouched]), "reference wrote points the oracle leaves untouched"
    assert np.array_equal(got_lib[written], got_ref[written]), "library differs from the reference kernel"
    if racy.any():
        n = int((got_lib[racy & (st == 1)] != got_ref[racy & (st == 1)]).sum())
        print(f"Ynp racy block row: {n} points differ from the reference (its missing barrier)")
