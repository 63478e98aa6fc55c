"""Failure detection without a GPU fault.

- The TMA stencil kernels' bounded mbarrier wait: a wait that nothing completes gives up after its
  limit, raises the device error flag, and the kernel returns; the context keeps computing correctly.
- The CH server: a request whose admission fails (an allocation failure injected on the host, a fake of
  the failing call) is marked failed with its reason while every other request completes with the same
  result as alone; requests that can never fit, or are malformed, are rejected at submit.
Nothing here traps, hangs or faults the GPU.
"""
import time

import numpy as np
import pytest

import custen_gb300 as cs
import oracle
from custen_gb300.buffers import DeviceBuffer
from custen_gb300.inputs import field, sentinel

pytestmark = pytest.mark.gpu


def test_bounded_wait_expires_and_context_survives(gpu):
    cs.device_error(clear=True)
    t0 = time.perf_counter()
    flags = cs.selftest_wait_expiry(1 << 12)
    assert time.perf_counter() - t0 < 5.0
    assert flags & 1, "the expired wait must raise bit 0"
    assert cs.device_error(clear=True) & 1
    assert cs.device_error() == 0
    # the context still computes: a TMA-staged stencil matches the oracle bit for bit, with no flag
    nx, ny = 256, 64
    inp = field(nx, ny, 3)
    w = np.random.default_rng(3).uniform(-1, 1, 9)
    pre = sentinel(nx, ny)
    d_in, d_out, d_w = DeviceBuffer.from_array(inp), DeviceBuffer.from_array(pre), DeviceBuffer.from_array(w)
    s = cs.Stencil(cs.XYP, nx, ny, d_out.ptr, d_in.ptr, d_w.ptr, H=3, L=1, R=1, V=3, T=1, B=1)
    s.compute()
    cs._check(cs.lib().custen_device_synchronize())
    got = d_out.download((ny, nx), np.float64)
    s.destroy()
    ref = pre.copy()
    oracle.stencil(cs.XYP, ref, inp, w, num_tiles=1, block_x=32, block_y=8, H=3, L=1, R=1, V=3, T=1, B=1)
    assert np.array_equal(got, ref)
    assert cs.device_error() == 0


def test_selftest_rejects_bad_limits(gpu):
    with pytest.raises(cs.CustenError):
        cs.selftest_wait_expiry(0)
    with pytest.raises(cs.CustenError):
        cs.selftest_wait_expiry(1 << 23)


def _alone(n, c0, steps):
    b = cs.CahnHilliardBatch([n])
    b.set_state(0, c0)
    b.step(steps, graph=False)
    out = b.state(0)[0]
    b.close()
    return out


@pytest.mark.parametrize("victim", [0, 2, 4])
def test_failed_request_is_isolated(gpu, victim):
    """An admission failure stays with its request: the others complete, bit-identical to alone."""
    reqs = [(64, 12, 0.0), (128, 10, 0.0), (96, 14, 0.0), (64, 8, 0.01), (128, 9, 0.02)]
    rng = np.random.default_rng(5)
    c0s = [rng.uniform(-0.1, 0.1, (n, n)) for n, _, _ in reqs]
    srv = cs.CahnHilliardServer(hbm_budget_bytes=1e9, chunk_steps=3)
    ids = [srv.submit(n, s, arrival=a, c0=c) for (n, s, a), c in zip(reqs, c0s)]
    srv.inject_failure(ids[victim])
    srv.run()
    for rid, (n, s, _), c in zip(ids, reqs, c0s):
        if rid == ids[victim]:
            assert srv.state(rid) == "failed"
            with pytest.raises(cs.CustenError, match="request failed: .*Allocating.*out of memory"):
                srv.result(rid)
            continue
        assert srv.state(rid) == "done"
        r = srv.result(rid)
        assert np.array_equal(r["field"], _alone(n, c, s)), f"request {rid} differs from its run alone"
        assert abs(r["mean_end"] - r["mean0"]) <= 1e-12
    st = srv.stats()
    assert st["steps"] == sum(s for k, (_, s, _) in enumerate(reqs) if k != victim)
    srv.close()


def test_every_request_failing_ends_the_run(gpu):
    srv = cs.CahnHilliardServer(hbm_budget_bytes=1e9, chunk_steps=2)
    ids = [srv.submit(64, 5, seed=k + 1) for k in range(3)]
    for rid in ids:
        srv.inject_failure(rid)
    srv.run()
    assert [srv.state(r) for r in ids] == ["failed"] * 3
    assert srv.stats()["steps"] == 0
    srv.close()


def test_request_above_the_budget_is_rejected_at_submit(gpu):
    srv = cs.CahnHilliardServer(hbm_budget_bytes=4 * 128 * 128 * 8, chunk_steps=2)
    with pytest.raises(cs.CustenError, match="above the server's HBM budget"):
        srv.submit(256, 4, seed=1)
    srv.close()


@pytest.mark.parametrize("n,steps", [(48, 4), (100, 4), (64, 0)])
def test_malformed_request_is_rejected(gpu, n, steps):
    srv = cs.CahnHilliardServer(hbm_budget_bytes=1e9)
    with pytest.raises(cs.CustenError, match="invalid request"):
        srv.submit(n, steps, seed=1)
    srv.close()
