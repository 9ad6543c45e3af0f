"""Serving traces for the request loop (phelm.Server / phg_serve_*).

A trace is a seeded list of requests with Poisson arrival times: a fraction
of Laplace solves with spherical-harmonic right-hand sides (l <= 10) and
otherwise short barotropic integrations from Rossby-Haurwitz + noise states,
mesh levels drawn uniformly.  ``run_trace`` submits each request at its
arrival time, collects the completions and reports latency percentiles
(arrival -> result on the host) and throughput.  Inputs come from small
per-(kind, level) pools of seeded fields (a request's input is read-only, so
pool entries are shared); every request gets its own output array.
"""
from __future__ import annotations

import time

import numpy as np

from . import fields, phelm

KIND_NAMES = {phelm.PHG_REQ_LAPLACE_SOLVE: "laplace_solve", phelm.PHG_REQ_BARVORTEX: "barvortex"}


def sh_basis(lat, lon, lmax: int):
    """Real orthonormal Y_lm, 1 <= l <= lmax, as a (n_modes x V) matrix and the degree of each row."""
    Y = fields.real_sph_harm(lmax, lat, lon)
    keys = [(l, m) for l in range(1, lmax + 1) for m in range(-l, l + 1)]
    return np.stack([Y[k] for k in keys]), np.array([l for l, _ in keys], dtype=np.float64)


def solve_inputs(lat, lon, count: int, seed: int, lmax: int = 10) -> np.ndarray:
    """count right-hand sides sum c_lm Y_lm (l = 1..lmax, c ~ N(0,1), coefficient norm 1)."""
    B, _ = sh_basis(lat, lon, lmax)
    c = np.random.default_rng(seed).standard_normal((count, B.shape[0]))
    c /= np.linalg.norm(c, axis=1, keepdims=True)
    return np.ascontiguousarray(c @ B)


def barvortex_inputs(lat, lon, count: int, seed: int, lmax_noise: int = 16, amp_rh: float = 0.1,
                     amp_noise: float = 1e-3) -> np.ndarray:
    """count stream functions Laplacian^{-1}(RH4 + noise), noise coefficients of norm amp_noise."""
    B, ls = sh_basis(lat, lon, lmax_noise)
    c = np.random.default_rng(seed).standard_normal((count, B.shape[0]))
    c *= amp_noise / np.linalg.norm(c, axis=1, keepdims=True)
    psi_rh = fields.rossby_haurwitz4(lat, lon, amp_rh) / -30.0
    return np.ascontiguousarray(psi_rh[None, :] + (c * (-1.0 / (ls * (ls + 1.0)))[None, :]) @ B)


def make_trace(n: int = 10000, rate: float = 2000.0, levels=(3, 4, 5, 6, 7), frac_solve: float = 0.6,
               steps: int = 10, pool: int = 16, seed: int = 2024):
    """Requests as (arrival_s, kind, level, steps, pool_index), sorted by arrival."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    kinds = np.where(rng.random(n) < frac_solve, phelm.PHG_REQ_LAPLACE_SOLVE, phelm.PHG_REQ_BARVORTEX)
    lv = rng.choice(np.asarray(levels), n)
    idx = rng.integers(0, pool, n)
    return [(float(t[i]), int(kinds[i]), int(lv[i]), steps if kinds[i] == phelm.PHG_REQ_BARVORTEX else 1,
             int(idx[i])) for i in range(n)]


def make_pools(trace, pool: int = 16, seed: int = 2024):
    """Input pools for every (kind, level) the trace uses."""
    need = sorted({(k, lv) for _, k, lv, _, _ in trace})
    meshes = {}
    pools = {}
    for kind, level in need:
        if level not in meshes:
            m = phelm.Mesh.sphere(level)
            meshes[level] = m.latlon()
        lat, lon = meshes[level]
        s = seed + 1000 * level + kind
        pools[(kind, level)] = (solve_inputs(lat, lon, pool, s) if kind == phelm.PHG_REQ_LAPLACE_SOLVE
                                else barvortex_inputs(lat, lon, pool, s))
    return pools


def run_trace(server: "phelm.Server", trace, pools, keep=None, time_scale: float = 1.0, stall_s: float = 300.0):
    """Submit every request at its arrival time; returns the statistics and,
    for the tags in ``keep``, the outputs."""
    n = len(trace)
    t_arr = np.zeros(n)
    done = np.zeros(n)
    status = np.zeros(n, dtype=np.int64)
    batch = np.zeros(n, dtype=np.int64)
    errors = {}
    kinds = np.array([r[1] for r in trace])
    levels = np.array([r[2] for r in trace])
    kept = {}
    got = 0

    def collect(wait):
        nonlocal got
        for c in server.poll(wait=wait):
            i = c["tag"]
            done[i] = c["t_done"]
            status[i] = c["status"]
            batch[i] = c["batch"]
            if c["status"]:
                key = f'{KIND_NAMES.get(c["kind"], c["kind"])} L{c["level"]}: {c["error"]}'
                errors[key] = errors.get(key, 0) + 1
            if keep is not None and i in keep:
                kept[i] = c["output"]
            got += 1

    t0 = server.clock()
    wall0 = time.perf_counter()
    for i, (ta, kind, level, steps, pi) in enumerate(trace):
        t_arr[i] = t0 + ta * time_scale
        while True:
            now = server.clock()
            if now >= t_arr[i]:
                break
            collect(0.0)
            gap = t_arr[i] - server.clock()
            if gap > 2e-4:
                time.sleep(min(gap, 1e-3) * 0.5)
        server.submit(kind, level, pools[(kind, level)][pi], steps=steps, tag=i)
    last, seen = time.perf_counter(), got
    while got < n:
        collect(0.5)
        if got != seen:
            last, seen = time.perf_counter(), got
        elif time.perf_counter() - last > stall_s:
            raise RuntimeError(f"serving trace stalled: {n - got} requests without a completion for {stall_s} s")
    wall = time.perf_counter() - wall0
    lat_ms = (done - t_arr) * 1e3
    ok = status == 0
    span = float(done.max() - t0) if n else 0.0

    def pct(x, q):
        return float(np.percentile(x, q)) if len(x) else None

    per_kind = {}
    for k, name in KIND_NAMES.items():
        sel = ok & (kinds == k)
        per_kind[name] = {"requests": int(sel.sum()), "p50_ms": pct(lat_ms[sel], 50), "p99_ms": pct(lat_ms[sel], 99),
                          "mean_batch": float(batch[sel].mean()) if sel.any() else None}
    per_level = {int(lv): {"requests": int((ok & (levels == lv)).sum()),
                           "p50_ms": pct(lat_ms[ok & (levels == lv)], 50),
                           "p99_ms": pct(lat_ms[ok & (levels == lv)], 99)} for lv in sorted(set(levels.tolist()))}
    n_solve = int((ok & (kinds == phelm.PHG_REQ_LAPLACE_SOLVE)).sum())
    n_steps = int(sum(trace[i][3] for i in range(n) if ok[i] and kinds[i] == phelm.PHG_REQ_BARVORTEX))
    stats = {
        "requests": n, "errors": int((~ok).sum()), "p50_ms": pct(lat_ms[ok], 50), "p99_ms": pct(lat_ms[ok], 99),
        "makespan_s": span, "wall_s": wall, "requests_per_s": float(ok.sum()) / span if span > 0 else None,
        "solves_per_s": n_solve / span if span > 0 else None,
        "barvortex_member_steps_per_s": n_steps / span if span > 0 else None,
        "per_kind": per_kind, "per_level": per_level, "error_kinds": errors,
    }
    return stats, kept
