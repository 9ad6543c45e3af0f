"""The request loop (phg_serve_*): continuous batching, admission by HBM budget,
per-request errors, and the same result for a request alone and in a mix.

Tolerance: solves run to 1e-12 relative residual here; a request served in a
batch of other members differs from the same request alone only by the
solver's rounding and stopping point, 1e-9 relative L2 (the tolerance of the
other solve and time-step tests).
"""
import time

import numpy as np
import pytest

from mke_gb300 import phelm, serve

pytestmark = pytest.mark.gpu

TOL = 1e-9
SOLVE, BV = phelm.PHG_REQ_LAPLACE_SOLVE, phelm.PHG_REQ_BARVORTEX


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def wait_for(srv, tags, timeout=120.0):
    got = {}
    t0 = time.time()
    while len(got) < len(tags):
        for c in srv.poll(wait=0.2):
            got[c["tag"]] = c
        assert time.time() - t0 < timeout, "requests did not complete"
    return got


def inputs(level, seed):
    lat, lon = phelm.Mesh.sphere(level).latlon()
    return serve.solve_inputs(lat, lon, 1, seed)[0], serve.barvortex_inputs(lat, lon, 1, seed)[0]


@pytest.fixture(scope="module")
def server():
    srv = phelm.Server(precision=phelm.PHG_FP64, hbm_budget_bytes=40e9, max_slots=8, solve_tol=1e-12,
                       step_tol=1e-12)
    yield srv
    srv.close()


def test_alone_vs_mix(server):
    F, psi = inputs(4, 11)
    server.submit(SOLVE, 4, F, tag=10**6)
    server.submit(BV, 4, psi, steps=3, tag=10**6 + 1)
    alone = wait_for(server, {10**6, 10**6 + 1})
    assert all(c["status"] == 0 for c in alone.values())
    a_s, a_b = alone[10**6]["output"], alone[10**6 + 1]["output"]

    # the same two requests in the middle of a mixed trace over levels 3..5
    trace = serve.make_trace(n=80, rate=400.0, levels=(3, 4, 5), frac_solve=0.5, steps=3, pool=4, seed=5)
    pools = serve.make_pools(trace, pool=4, seed=5)
    pools[(SOLVE, 4)] = np.vstack([pools.get((SOLVE, 4), np.zeros((0, F.size))), F[None, :]])
    pools[(BV, 4)] = np.vstack([pools.get((BV, 4), np.zeros((0, psi.size))), psi[None, :]])
    mid = trace[40][0]
    trace[40] = (mid, SOLVE, 4, 1, len(pools[(SOLVE, 4)]) - 1)
    trace[41] = (trace[41][0], BV, 4, 3, len(pools[(BV, 4)]) - 1)
    stats, kept = serve.run_trace(server, trace, pools, keep={40, 41})
    assert stats["errors"] == 0, stats["error_kinds"]
    assert rel(kept[40], a_s) <= TOL
    assert rel(kept[41], a_b) <= TOL
    # requests were batched with others
    assert stats["per_kind"]["barvortex"]["mean_batch"] > 1.0

    # and both agree with the direct library calls
    m = phelm.Mesh.sphere(4)
    ops = phelm.Operators(m, phelm.PHG_FP64, tol=1e-12)
    assert rel(phelm.SphereLaplace(ops).solve(F), a_s) <= TOL
    lat, _ = m.latlon()
    bv = phelm.BarVortex(ops, tau=1e-3, sigma=1.6e-2, mu=8e-5, theta=0.5, picard_iters=3, coriolis=np.sin(lat))
    u = psi.copy()
    for _ in range(3):
        u = bv.calc(u)
    assert rel(u, a_b) <= TOL


def test_member_joins_running_batch(server):
    _, psi_a = inputs(5, 21)
    _, psi_b = inputs(5, 22)
    server.preload(BV, 5)
    server.submit(BV, 5, psi_a, steps=40, tag=1)
    time.sleep(0.02)
    server.submit(BV, 5, psi_b, steps=2, tag=2)
    got = wait_for(server, {1, 2})
    a, b = got[1], got[2]
    assert a["status"] == 0 and b["status"] == 0
    # b entered while a was stepping and left first
    assert b["t_admit"] < a["t_done"] and b["t_done"] < a["t_done"]
    assert b["batch"] == 2
    # a's result does not depend on b having shared its launches
    server.submit(BV, 5, psi_a, steps=40, tag=3)
    alone = wait_for(server, {3})[3]
    assert rel(a["output"], alone["output"]) <= TOL


def test_lanes_overlap(server):
    """Requests of different levels are served concurrently."""
    _, p5 = inputs(5, 31)
    _, p6 = inputs(6, 32)
    server.preload(BV, 6)
    server.submit(BV, 6, p6, steps=6, tag=100)
    server.submit(BV, 5, p5, steps=6, tag=101)
    got = wait_for(server, {100, 101})
    x, y = got[100], got[101]
    assert x["status"] == 0 and y["status"] == 0
    assert max(x["t_admit"], y["t_admit"]) < min(x["t_done"], y["t_done"])


def test_request_errors():
    srv = phelm.Server(precision=phelm.PHG_MIXED, hbm_budget_bytes=1e6, max_slots=4)
    try:
        F, _ = inputs(3, 1)
        srv.submit(SOLVE, 0, F, tag=1)            # no such level
        srv.submit(BV, 3, F, steps=0, tag=2)      # no steps
        srv.submit(SOLVE, 3, F, tag=3)            # the lane needs more than 1 MB
        got = wait_for(srv, {1, 2, 3})
        assert got[1]["status"] == 1 and got[2]["status"] == 1
        assert got[3]["status"] == 6
        assert srv.stats()["bytes_in_use"] <= 1e6
    finally:
        srv.close()


def test_budget_evicts_idle_lane():
    """A budget that holds one lane at a time: the idle lane is closed for the next."""
    F3, _ = inputs(3, 2)
    F4, _ = inputs(4, 3)
    probe = phelm.Server(precision=phelm.PHG_FP64, hbm_budget_bytes=40e9, max_slots=2, solve_tol=1e-12)
    try:
        probe.preload(SOLVE, 3)
        b3 = probe.stats()["bytes_in_use"]
        probe.preload(SOLVE, 4)
        b4 = probe.stats()["bytes_in_use"] - b3
    finally:
        probe.close()
    budget = 1.02 * max(b3, b4)
    assert budget < b3 + b4
    srv = phelm.Server(precision=phelm.PHG_FP64, hbm_budget_bytes=budget, max_slots=2, solve_tol=1e-12)
    try:
        srv.submit(SOLVE, 3, F3, tag=1)
        a = wait_for(srv, {1})[1]
        srv.submit(SOLVE, 4, F4, tag=2)
        b = wait_for(srv, {2})[2]
        assert a["status"] == 0 and b["status"] == 0, (a["status"], b["status"])
        st = srv.stats()
        assert st["bytes_in_use"] <= budget and st["lanes"] == 1
    finally:
        srv.close()


def test_full_lane_runs_captured_steps():
    """A barotropic lane whose slots are all taken advances its members by
    several steps per call from the captured step graph (one graph per member
    count); every request's result equals the same integration by direct
    library calls.  Six 5-step requests on two slots: the lane is full
    throughout, members leave and join between runs."""
    level, steps = 3, 5
    m = phelm.Mesh.sphere(level)
    lat, lon = m.latlon()
    psi = serve.barvortex_inputs(lat, lon, 6, 21)
    srv = phelm.Server(precision=phelm.PHG_MIXED, hbm_budget_bytes=20e9, max_slots=2, solve_tol=1e-12,
                       step_tol=1e-12)
    try:
        for k in range(6):
            srv.submit(BV, level, psi[k], steps=steps + (k % 2), tag=k)
        got = wait_for(srv, set(range(6)))
    finally:
        srv.close()
    ops = phelm.Operators(m, phelm.PHG_MIXED, tol=1e-12)
    conf = dict(tau=1e-3, sigma=1.6e-2, mu=8e-5, k1=1.0, k2=1.0, theta=0.5, picard_iters=3)
    bv = phelm.BarVortex(ops, coriolis=np.sin(lat), **conf)
    z = np.zeros(m.outer_size)
    for k in range(6):
        assert got[k]["status"] == 0, got[k]
        x = psi[k].copy()
        for _ in range(steps + (k % 2)):
            x = bv.calc(x, z, z)
        assert rel(got[k]["output"], x) <= TOL, k


@pytest.mark.parametrize("pack", ["5", "0"])
def test_packed_laplace_levels(pack, monkeypatch):
    """Laplace requests of levels 3..5 share one lane and one multi-level
    launch per turn (PHG_SERVE_PACK=5, the default); with packing off each
    level has its own lane.  Results equal the direct solves either way, and a
    packed turn holds members of several levels."""
    monkeypatch.setenv("PHG_SERVE_PACK", pack)
    levels, per = (3, 4, 5), 4
    Fs = {lv: serve.solve_inputs(*phelm.Mesh.sphere(lv).latlon(), per, 70 + lv) for lv in levels}
    srv = phelm.Server(precision=phelm.PHG_MIXED, hbm_budget_bytes=40e9, max_slots=8, solve_tol=1e-12)
    try:
        for lv in levels:
            srv.preload(SOLVE, lv)
        lanes = srv.stats()["lanes"]
        for j in range(per):
            for lv in levels:
                srv.submit(SOLVE, lv, Fs[lv][j], tag=100 * lv + j)
        got = wait_for(srv, {100 * lv + j for lv in levels for j in range(per)})
    finally:
        srv.close()
    assert lanes == (1 if pack == "5" else 3)
    for lv in levels:
        ops = phelm.Operators(phelm.Mesh.sphere(lv), phelm.PHG_MIXED, tol=1e-12)
        want = phelm.SphereLaplace(ops).solve_batch(Fs[lv])
        for j in range(per):
            c = got[100 * lv + j]
            assert c["status"] == 0, c
            assert rel(c["output"], want[j]) <= TOL, (lv, j)
    if pack == "5":
        # a turn of more than `per` members holds more than one level
        assert max(c["batch"] for c in got.values()) > per


def test_packed_lane_closes_idle_level(monkeypatch):
    """A packed Laplace lane under a budget that holds one level at a time:
    the level opened first is closed (least recently used, idle) to make room
    for the next, and both requests complete."""
    monkeypatch.setenv("PHG_SERVE_PACK", "5")
    F3, _ = inputs(3, 4)
    F4, _ = inputs(4, 5)
    probe = phelm.Server(precision=phelm.PHG_FP64, hbm_budget_bytes=40e9, max_slots=2, solve_tol=1e-12)
    try:
        probe.preload(SOLVE, 3)
        b3 = probe.stats()["bytes_in_use"]
        probe.preload(SOLVE, 4)
        b4 = probe.stats()["bytes_in_use"] - b3
    finally:
        probe.close()
    budget = 1.02 * max(b3, b4)
    assert budget < b3 + b4
    srv = phelm.Server(precision=phelm.PHG_FP64, hbm_budget_bytes=budget, max_slots=2, solve_tol=1e-12)
    try:
        srv.submit(SOLVE, 3, F3, tag=1)
        a = wait_for(srv, {1})[1]
        srv.submit(SOLVE, 4, F4, tag=2)
        b = wait_for(srv, {2})[2]
        assert a["status"] == 0 and b["status"] == 0, (a, b)
        st = srv.stats()
        assert st["bytes_in_use"] <= budget and st["lanes"] == 1
    finally:
        srv.close()
    ops = phelm.Operators(phelm.Mesh.sphere(4), phelm.PHG_FP64, tol=1e-12)
    assert rel(b["output"], phelm.SphereLaplace(ops).solve(F4)) <= TOL
