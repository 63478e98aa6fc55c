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


def test_served_2048_request_in_mix_equals_alone(gpu):
    """A 2048^2 request served in a mix of smaller ones that arrive while it runs: bit-identical to its run
    alone, mass conserved; the smaller requests likewise."""
    reqs = [(2048, 12, 0.0), (512, 20, 0.0), (128, 30, 0.01), (1024, 8, 0.02), (256, 16, 0.05)]
    rng = np.random.default_rng(78)
    c0s = [rng.uniform(-0.1, 0.1, (n, n)) for n, _, _ in reqs]
    srv = cs.CahnHilliardServer(hbm_budget_bytes=4e9, chunk_steps=4)
    ids = [srv.submit(n, s, arrival=a, c0=c) for (n, s, a), c in zip(reqs, c0s)]
    srv.run()
    st = srv.stats()
    assert st["steps"] == sum(s for _, s, _ in reqs)
    assert st["max_active"] >= 2, "requests should overlap on the device"
    for rid, (n, s, a), c in zip(ids, reqs, c0s):
        r = srv.result(rid)
        assert np.array_equal(r["field"], _alone(n, c, s)), f"request {rid} ({n}^2) differs from its run alone"
        assert abs(r["mean_end"] - r["mean0"]) <= 1e-12
    srv.close()


def test_budget_limits_resident_set(gpu):
    """A budget that holds two 128^2 grids at a time: four requests still all complete."""
    per_grid = 4 * 128 * 128 * 8 + 2 * 128 * 8
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


def _batch_steps(n, c0, steps):
    b = cs.CahnHilliardBatch([n])
    b.set_state(0, c0)
    b.step(steps, graph=False)
    out = b.state(0)
    b.close()
    return out


def _times(n, steps, every, lx=2 * np.pi, t0=0.0):
    """Snapshot times as the reference accumulates them: time += dt after every step."""
    dt = 0.1 * (lx / n)
    t, out = t0, []
    for k in range(1, steps + 1):
        t += dt
        if k % every == 0:
            out.append(t)
    return out


def test_snapshots_and_resume(gpu, tmp_path):
    """Snapshots every 5 steps carry the batch's fields bit for bit under the reference's file names; a
    request resumed from the step-10 snapshot ends bit-identical to the uninterrupted one."""
    n, steps = 64, 20
    c0 = np.random.default_rng(9).uniform(-0.1, 0.1, (n, n))
    a_dir, b_dir = tmp_path / "a", tmp_path / "b"
    a_dir.mkdir()
    b_dir.mkdir()
    srv = cs.CahnHilliardServer(hbm_budget_bytes=1e9, chunk_steps=8)
    rid = srv.submit(n, steps, c0=c0)
    other = srv.submit(96, 13, seed=4)                       # a neighbour without snapshots
    srv.snapshots(rid, 5, a_dir)
    srv.run()
    assert srv.snapshots_written(rid) == 4 and srv.snapshots_written(other) == 0
    times = _times(n, steps, 5)
    for k, t in enumerate(times, start=1):
        p = a_dir / cs.snapshot_name(t)
        assert p.exists(), p.name
        cur, old = _batch_steps(n, c0, 5 * k)
        assert np.array_equal(cs.h5_read(p, "c"), cur) and np.array_equal(cs.h5_read(p, "c_old"), old)
        assert cs.h5_read(p, "t")[0, 0] == t
    final = srv.result(rid)["field"]
    srv.close()

    srv = cs.CahnHilliardServer(hbm_budget_bytes=1e9, chunk_steps=3)
    rb = srv.submit_snapshot(a_dir / cs.snapshot_name(times[1]), 10)
    srv.snapshots(rb, 10, b_dir)
    srv.run()
    assert np.array_equal(srv.result(rb)["field"], final)
    assert (b_dir / cs.snapshot_name(times[3])).exists()     # the same time as the uninterrupted run's
    srv.close()


def test_resume_from_a_reference_style_snapshot_in_the_server(gpu, tmp_path):
    """A file holding only "c" (the reference's snapshot) starts a fresh request from it."""
    n = 64
    c = np.random.default_rng(12).uniform(-0.1, 0.1, (n, n))
    p = tmp_path / cs.snapshot_name(0.0)
    cs.h5_write(p, {"c": c})
    srv = cs.CahnHilliardServer(hbm_budget_bytes=1e9, chunk_steps=4)
    rid = srv.submit_snapshot(p, 7)
    srv.run()
    assert np.array_equal(srv.result(rid)["field"], _batch_steps(n, c, 7)[0])
    srv.close()


def test_failed_snapshot_write_fails_only_its_request(gpu, tmp_path):
    srv = cs.CahnHilliardServer(hbm_budget_bytes=1e9, chunk_steps=4)
    bad = srv.submit(64, 10, seed=1)
    good = srv.submit(64, 10, seed=2)
    srv.snapshots(bad, 5, tmp_path / "missing" / "dir")
    srv.run()
    assert srv.state(bad) == "failed" and srv.state(good) == "done"
    with pytest.raises(cs.CustenError, match="Writing a snapshot"):
        srv.result(bad)
    r = srv.result(good)
    assert abs(r["mean_end"] - r["mean0"]) <= 1e-12
    srv.close()
