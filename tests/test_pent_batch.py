"""Batched pentadiagonal factorisation and solve (cuPentBatch's pentFactorBatch / pentSolveBatch) on the
GPU: bit-identical to the oracle and to the reference's own kernels; the inverted-pivot solve within a
stated tolerance (GPU)."""
import numpy as np
import pytest

import custen_gb300 as cs
import oracle
from custen_gb300.buffers import DeviceBuffer
from custen_gb300.inputs import pent_system
from tests.helpers import pent_dense_apply

pytestmark = pytest.mark.gpu

SHAPES = [(4, 1), (5, 130), (32, 129), (64, 1000), (257, 300)]


def run_lib(m, batch, seed, rcp=False):
    sysm = pent_system(m, batch, seed)
    bufs = [DeviceBuffer.from_array(a) for a in sysm]
    cs.pent_factor_batch(*[b.ptr for b in bufs[:5]], m, batch)
    if rcp:
        cs.pent_invert_pivots(bufs[2].ptr, m, batch)
    cs.pent_solve_batch(*[b.ptr for b in bufs], m, batch, inverted_pivots=rcp)
    cs._check(cs.lib().custen_device_synchronize())
    return sysm, [b.download((m, batch), np.float64) for b in bufs]


@pytest.mark.parametrize("m,batch", SHAPES)
def test_factor_and_solve_bit_identical_to_oracle(gpu, m, batch):
    sysm, got = run_lib(m, batch, m + batch)
    f = oracle.pent_factor(*sysm[:5])
    for k, name in enumerate(("ds", "dl", "d", "du", "dw")):
        assert np.array_equal(got[k], f[k]), name
    assert np.array_equal(got[5], oracle.pent_solve(f, sysm[5]))


@pytest.mark.parametrize("m,batch", [(32, 129), (257, 300)])
def test_bit_identical_to_reference_kernels(gpu, m, batch):
    if not oracle.ReferenceCahnHilliardGPU.available():
        pytest.skip("reference CH cubin not present")
    sysm, got = run_lib(m, batch, 7)
    bufs = [DeviceBuffer.from_array(a) for a in sysm]
    oracle.reference_pent(True, [b.ptr for b in bufs[:5]], m, batch)
    oracle.reference_pent(False, [b.ptr for b in bufs], m, batch)
    for k in range(6):
        assert np.array_equal(got[k], bufs[k].download((m, batch), np.float64)), k


@pytest.mark.parametrize("m,batch", [(5, 64), (257, 300)])
def test_inverted_pivot_solve(gpu, m, batch):
    """Multiplications by inverted pivots instead of divisions: the solution satisfies the systems and
    agrees with the exact solve to a few units in the last place."""
    sysm, got = run_lib(m, batch, 3, rcp=True)
    _, exact = run_lib(m, batch, 3)
    x = got[5]
    assert np.abs(pent_dense_apply(*sysm[:5], x) - sysm[5]).max() < 1e-13
    assert np.abs(x - exact[5]).max() <= 1e-14 * np.abs(exact[5]).max()


def test_rejects_bad_arguments(gpu):
    buf = DeviceBuffer(64)
    with pytest.raises(cs.CustenError):
        cs.pent_factor_batch(buf.ptr, buf.ptr, buf.ptr, buf.ptr, buf.ptr, 3, 1)
    with pytest.raises(cs.CustenError):
        cs.pent_solve_batch(buf.ptr, buf.ptr, buf.ptr, buf.ptr, buf.ptr, None, 8, 1)
