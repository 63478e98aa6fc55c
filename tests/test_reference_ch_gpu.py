"""The reference's own Cahn-Hilliard GPU program (device code compiled unchanged, host loop restated in
oracle/ref_ch_runner.cpp) against the serial oracle, and the library's batched solver against it (GPU)."""
import numpy as np
import pytest

import custen_gb300 as cs
import oracle

pytestmark = pytest.mark.gpu


def _need_ref():
    if not oracle.ReferenceCahnHilliardGPU.available():
        pytest.skip("reference CH cubin not present")


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n", [64, 128])
def test_reference_gpu_program_matches_serial_oracle(gpu, n):
    _need_ref()
    c0 = np.random.default_rng(n).uniform(-0.1, 0.1, (n, n))
    ref = oracle.ReferenceCahnHilliardGPU(c0)
    ref.step(40)
    cur, old = ref.state()
    ref.close()
    ora = oracle.CHOracle(c0)
    ora.step(40)
    ocur, oold = ora.fields()
    assert rel_l2(cur, ocur) <= 1e-12 and rel_l2(old, oold) <= 1e-12


def test_library_batch_matches_reference_gpu_program(gpu):
    """Grids of two sizes in one batch against the reference program run one grid at a time."""
    _need_ref()
    sizes = [64, 192]
    c0s = [np.random.default_rng(7 + k).uniform(-0.1, 0.1, (n, n)) for k, n in enumerate(sizes)]
    b = cs.CahnHilliardBatch(sizes)
    for k, c0 in enumerate(c0s):
        b.set_state(k, c0)
    b.step(60)
    b.synchronize()
    for k, (n, c0) in enumerate(zip(sizes, c0s)):
        ref = oracle.ReferenceCahnHilliardGPU(c0)
        ref.step(60)
        rcur, rold = ref.state()
        ref.close()
        cur, old = b.state(k)
        assert rel_l2(cur, rcur) <= 1e-10, n
        assert rel_l2(old, rold) <= 1e-10, n
    b.close()
