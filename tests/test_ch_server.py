"""Cahn-Hilliard serving (GPU): continuous batching with HBM-budget admission.

Requests arriving while others run are admitted between chunks and advance together with them; each
result must be the same alone and in the mix (bit-identical: the per-grid arithmetic does not depend
on what else is resident), mass must be conserved, and the budget must bound the resident set.
"""
import numpy as np
import pytest

import custen_gb300 as cs

pytestmark = pytest.mark.gpu


def _alone(n, c0, steps):
    b = cs.CahnHilliardBatch([n])
    b.set_state(0, c0)
    b.step(steps, graph=False)
    out = b.state(0)[0]
    b.close()
    return out


def test_served_results_equal_alone(gpu):
    reqs = [(64, 30, 0.0), (128, 20, 0.0), (96, 40, 0.02), (64, 12, 0.05), (128, 25, 0.1), (64, 9, 0.3)]
    rng = np.random.default_rng(77)
    c0s = [rng.uniform(-0.1, 0.1, (n, n)) for n, _, _ in reqs]
    srv = cs.CahnHilliardServer(hbm_budget_bytes=1e9, chunk_steps=4)
    ids = [srv.submit(n, s, arrival=a, c0=c) for (n, s, a), c in zip(reqs, c0s)]
    srv.run()
    st = srv.stats()
    assert st["steps"] == sum(s for _, s, _ in reqs)
    assert st["max_active"] >= 2, "requests should overlap on the device"
    for rid, (n, s, a), c in zip(ids, reqs, c0s):
        r = srv.result(rid)
        assert r["done"] >= r["admit"] >= r["arrival"] - 1e-9
        assert np.array_equal(r["field"], _alone(n, c, s)), f"request {rid} differs from its run alone"
        assert abs(r["mean_end"] - r["mean0"]) <= 1e-12
    srv.close()


def test_budget_limits_resident_set(gpu):
    """A budget that holds two 128^2 grids at a time: four requests still all complete."""
    per_grid = 3 * 128 * 128 * 8 + 2 * 128 * 8
    table = (7 * 126 + 42) * 8
    srv = cs.CahnHilliardServer(hbm_budget_bytes=2 * per_grid + table + 1024, chunk_steps=3, keep_results=False)
    for k in range(4):
        srv.submit(128, 10 + 3 * k, arrival=0.0, seed=k + 1)
    srv.run()
    st = srv.stats()
    assert st["max_active"] <= 2
    assert st["peak_bytes"] <= 2 * per_grid + table + 1024
    for k in range(4):
        r = srv.result(k, field=False)
        assert abs(r["mean_end"] - r["mean0"]) <= 1e-12
    srv.close()


def test_seeded_initial_field_is_uniform(gpu):
    srv = cs.CahnHilliardServer(chunk_steps=1)
    rid = srv.submit(64, 1, seed=123)
    srv.run()
    r = srv.result(rid)
    assert abs(r["mean0"]) < 0.01
    assert np.abs(r["field"]).max() < 0.2
    srv.close()
