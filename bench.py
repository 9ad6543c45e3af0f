#!/usr/bin/env python
"""Benchmark: barotropic-vorticity (barvortex) steps/s on an icosahedral
level-6 sphere mesh (40,962 points), mixed precision vs FP64, on GB300.

Workload (one "step" = one BarVortex::calc): tau = 1e-3, theta = 0.5,
3 Picard iterations, sigma = 1.6e-2, mu = 8e-5, k1 = k2 = 1, l + h = sin(lat)
(2 Omega = 1), zero boundary; the initial stream function is the inverse
Laplacian of a wavenumber-4 Rossby-Haurwitz vorticity (amplitude 0.1) plus
seeded spherical-harmonic noise (l <= 20, amplitude 1e-3).  Every linear
solve runs to a relative residual of 1e-10.

Arms: the default arm times the GB300 library through its C ABI; ``--impl
reference`` times the reference algorithm on the host cores (the C oracle,
the reference's own sources cannot run on this machine) on the same workload.
Multi-GPU runs are independent replicas (one trajectory per GPU, no
collective): the path does not shard at this size.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

LEVEL = 6
CONF = dict(tau=1e-3, sigma=1.6e-2, mu=8e-5, k1=1.0, k2=1.0, theta=0.5, picard_iters=3)
SEED = 2024
METRIC = "level-6 barvortex steps/s, mixed vs FP64 at 1e-10 rel err; serve p50/p99 ms"
TOL = 1e-11  # every solve: relative residual <= 1e-11: within the metric's 1e-10 per-solve bound and, unlike
             # 1e-10 itself, within 1e-8 of the reference's 100-step level-6 state (test_gpu_trajectory)
STRICT_TOL = 1e-12  # the same single-trajectory steps at a tighter tolerance, reported beside


def dist_env():
    from mke_gb300 import replicas
    return replicas.env()


class ClockSampler:
    """nvidia-smi SM clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def tune_in_child(level: int, precision: str, members: int) -> list:
    """Autotune (phg_ops_autotune) for a level / precision / ensemble size in a
    child process and load the saved shape table here.  Tuning in this
    process would leave its freed scratch behind the later allocations, which
    measurably moved the step's buffers (L6 x 32 ensemble step 22.0 -> 23.0 ms
    with identical shapes); a table tuned elsewhere and loaded does not.
    Returns the "chose ..." lines of the tuner's report."""
    import subprocess
    import tempfile
    from mke_gb300 import phelm
    fd, path = tempfile.mkstemp(suffix=".tune")
    os.close(fd)
    code = ("import json, sys; sys.path.insert(0, %r); from mke_gb300 import phelm; import bench; "
            "m = phelm.Mesh.sphere(%d); "
            "o = phelm.Operators(m, phelm.PHG_MIXED if %r == 'mixed' else phelm.PHG_FP64, restart=30, tol=%r); "
            "rep = o.autotune(%d); phelm.tune_save(%r); print(json.dumps(bench.chosen(rep)))"
            % (HERE, level, precision, TOL, members, path))
    # the child tunes on this rank's GPU, outside the process group
    env = dict(os.environ)
    local = int(os.environ.get("LOCAL_RANK", "0"))
    vis = [d for d in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if d.strip()]
    env["CUDA_VISIBLE_DEVICES"] = vis[local] if local < len(vis) else (vis[0] if vis else str(local))
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "LOCAL_WORLD_SIZE", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    try:
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=HERE, timeout=600,
                           env=env)
        if r.returncode != 0:
            raise RuntimeError(f"autotune child failed: {r.stderr[-2000:]}")
        phelm.tune_load(path)
        return json.loads(r.stdout.strip().splitlines()[-1])
    finally:
        os.unlink(path)


def chosen(report: str) -> list:
    """The "chose ..." lines of an autotuner report."""
    return [ln[6:] for ln in report.splitlines() if ln.startswith("chose ")]


def initial_state(mesh):
    from mke_gb300 import fields
    lat, lon = mesh.latlon()
    psi, _ = fields.barvortex_initial(lat, lon, seed=SEED)
    return psi, np.sin(lat)


def run_strict(mesh, psi0, cor, dev, stream, flush, steps: int, tol: float = STRICT_TOL):
    """Single-trajectory steps/s of both precisions with every solve to `tol`
    (graph-replayed steps, L2 flushed before each, CUDA events on the
    stream): the headline workload at a tighter solve tolerance."""
    import torch
    from mke_gb300 import phelm
    out = {}
    zb = torch.zeros(max(mesh.outer_size, 1), dtype=torch.float64, device=dev)
    for name, prec in (("mixed", phelm.PHG_MIXED), ("fp64", phelm.PHG_FP64)):
        ops = phelm.Operators(mesh, prec, restart=30, tol=tol, max_iter=20000)
        bv = phelm.BarVortex(ops, coriolis=cor, **CONF)
        u = torch.tensor(psi0, dtype=torch.float64, device=dev)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        with torch.cuda.stream(stream):
            bv.run(u, 3, zb, zb, stream=stream)
            for e0, e1 in ev:
                flush.zero_()
                e0.record(stream)
                bv.run(u, 1, zb, zb, stream=stream)
                e1.record(stream)
        stream.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in ev) / steps
        st = bv.last_stats()
        out[name] = {"steps_per_s": 1000.0 / ms, "worst_relres": st["worst_relres"]}
        del bv, ops
    return out


def run_ours(args, ws, rank, local):
    import torch
    from mke_gb300 import phelm

    from mke_gb300 import replicas
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    replicas.init("nccl", device=dev)   # replicas only: a collective for the timings, none on the data path
    barrier = replicas.barrier

    mesh = phelm.Mesh.sphere(args.level)
    psi0, cor = initial_state(mesh)
    V, os_ = mesh.size, mesh.outer_size
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # 256 MB > L2 (129 MB)

    tuned = {}

    def make(prec):
        ops = phelm.Operators(mesh, prec, restart=30, tol=args.tol, max_iter=20000)
        if not args.no_tune:
            pname = 'mixed' if prec == phelm.PHG_MIXED else 'fp64'
            tuned[f"L{args.level}x1_{pname}"] = tune_in_child(args.level, pname, 1)
        return ops, phelm.BarVortex(ops, coriolis=cor, **CONF)

    results = {}
    zb = torch.zeros(max(os_, 1), dtype=torch.float64, device=dev)
    for name, prec in (("mixed", phelm.PHG_MIXED), ("fp64", phelm.PHG_FP64)):
        ops, bv = make(prec)
        u = torch.tensor(psi0, dtype=torch.float64, device=dev)
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                bv.calc(u, zb, zb, out=u, stream=stream)
        stream.synchronize()
        u = torch.tensor(psi0, dtype=torch.float64, device=dev)
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        clocks = ClockSampler(local) if name == "mixed" else None
        if clocks:
            clocks.start()
        ops.profile(True)
        k0 = phelm.kernel_launches()
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.zero_()
                starts[k].record(stream)
                bv.calc(u, zb, zb, out=u, stream=stream)
                ends[k].record(stream)
        torch.cuda.synchronize()
        barrier()
        wall = time.perf_counter() - t0
        launches = phelm.kernel_launches() - k0 - 0
        prof = ops.profile_read(2)          # the Laplacian solves: gmres_kernel (the dominant kernel)
        prof_all = ops.profile_read()       # every solver launch (gmres_kernel + cheb_kernel)
        ops.profile(False)
        dev_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
        st = bv.last_stats()
        eager = {"ms_per_step": dev_ms / args.steps, "wall_s": wall, "launches": launches, "state": u.cpu().numpy()}
        # the same steps replayed from one captured CUDA graph (phg_barvortex_run)
        u = torch.tensor(psi0, dtype=torch.float64, device=dev)
        u0 = u.clone()
        with torch.cuda.stream(stream):
            bv.run(u, max(args.warmup, 2), zb, zb, stream=stream)   # captures for this state buffer
            u.copy_(u0)
        stream.synchronize()
        bv.last_stats()
        k0 = phelm.kernel_launches()
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.zero_()
                starts[k].record(stream)
                bv.run(u, 1, zb, zb, stream=stream)
                ends[k].record(stream)
        torch.cuda.synchronize()
        barrier()
        gwall = time.perf_counter() - t0
        glaunches = phelm.kernel_launches() - k0
        gst = bv.last_stats()
        graph = {"ms_per_step": sum(s.elapsed_time(e) for s, e in zip(starts, ends)) / args.steps,
                 "wall_s": gwall, "launches": glaunches, "state": u.cpu().numpy()}
        if not np.array_equal(graph["state"], eager["state"]):
            raise RuntimeError("graph-replayed steps differ from the steps enqueued kernel by kernel")
        best = graph if graph["ms_per_step"] < eager["ms_per_step"] else eager
        results[name] = {"ms_per_step": best["ms_per_step"], "wall_s": best["wall_s"], "prof": prof,
                         "prof_all": prof_all,
                         "launches": best["launches"], "state": best["state"], "stats": st,
                         "path": "graph" if best is graph else "eager",
                         "eager_ms": eager["ms_per_step"], "graph_ms": graph["ms_per_step"],
                         "worst_relres_graph": gst["worst_relres"],
                         "clocks": clocks.stop() if clocks else None}
        # end-to-end through the C ABI with host buffers (H2D/D2H every step)
        if name == "mixed":
            uh = psi0.copy()
            zh = np.zeros(max(os_, 1))
            out = np.empty_like(uh)
            bv.calc(uh, zh, zh, out=out)  # warm
            t1 = time.perf_counter()
            for _ in range(args.steps):
                bv.calc(uh, zh, zh, out=out)
                uh, out = out, uh
            e2e = time.perf_counter() - t1
            # host arrays through the captured step: copy in, replay, copy back, check
            ug = psi0.copy()
            bv.run(ug, 2, zh, zh)   # captures for the staged host arguments
            t1 = time.perf_counter()
            for _ in range(args.steps):
                bv.run(ug, 1, zh, zh)
            e2e_graph = time.perf_counter() - t1
            results[name]["e2e_s"] = min(e2e, e2e_graph)
            results[name]["e2e_eager_s"] = e2e
            results[name]["e2e_graph_s"] = e2e_graph
        del bv, ops

    strict = run_strict(mesh, psi0, cor, dev, stream, flush, args.steps) if args.tol != STRICT_TOL else None

    # batched ensembles: 256 members on level 5 (the ensemble workload), and 32 on level 6
    batched = {}
    if not args.no_batch:
        from mke_gb300 import fields
        for lvl, B in ((5, 256), (args.level, 32)):
            bm = mesh if lvl == args.level else phelm.Mesh.sphere(lvl)
            blat, blon = bm.latlon()
            states = np.stack([fields.barvortex_initial(blat, blon, seed=SEED + k, lmax_noise=16)[0] for k in range(B)])
            row = {"level": lvl, "members": B}
            for name, prec in (("mixed", phelm.PHG_MIXED), ("fp64", phelm.PHG_FP64)):
                bops = phelm.Operators(bm, prec, restart=30, tol=args.tol)
                if not args.no_tune:
                    tuned[f"L{lvl}x{B}_{name}"] = tune_in_child(lvl, name, B)
                bbv = phelm.BarVortex(bops, coriolis=np.sin(blat), **CONF)
                U = torch.tensor(states, dtype=torch.float64, device=dev)
                zB = torch.zeros((B, max(bm.outer_size, 1)), dtype=torch.float64, device=dev)
                with torch.cuda.stream(stream):
                    bbv.calc_batch(U, zB, zB, out=U, stream=stream)
                    stream.synchronize()
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    nb = 10   # steps per timing (the inputs exceed L2 at these sizes)
                    flush.zero_()
                    e0.record(stream)
                    for _ in range(nb):
                        bbv.calc_batch(U, zB, zB, out=U, stream=stream)
                    e1.record(stream)
                    stream.synchronize()
                    eager_ms = e0.elapsed_time(e1) / nb
                    # captured step, replayed (the inputs exceed L2 at these sizes)
                    bbv.run(U, 2, zB, zB, stream=stream)
                    stream.synchronize()
                    flush.zero_()
                    e0.record(stream)
                    bbv.run(U, nb, zB, zB, stream=stream)
                    e1.record(stream)
                stream.synchronize()
                bst = bbv.last_stats()
                graph_ms = e0.elapsed_time(e1) / nb
                bms = min(eager_ms, graph_ms)
                row[name] = {"member_steps_per_s": B * 1000.0 / bms, "ms_per_step": bms, "eager_ms": eager_ms,
                             "graph_ms": graph_ms, "worst_relres": bst["worst_relres"],
                             "state": U.cpu().numpy()}
                del bbv, bops
            row["mixed_over_fp64"] = row["mixed"]["member_steps_per_s"] / row["fp64"]["member_steps_per_s"]
            # the same members, the same 1 + 2 + 2 nb steps in both precisions
            a, b = row["mixed"].pop("state"), row["fp64"].pop("state")
            row["steps_compared"] = 3 + 2 * nb
            row["rel_err_vs_fp64"] = float(max(np.linalg.norm(a[k] - b[k]) / np.linalg.norm(b[k]) for k in range(B)))
            batched[f"L{lvl}x{B}"] = row

    # two-layer baroclinic steps, level 6 (the reference's baroclin configuration)
    baroclin = None if args.no_baroclin else run_baroclin(args.level, 20)

    # operator apply at a streaming size (level 8, 64 FP32 vectors; one FP64 vector)
    spmv = None if args.no_spmv else run_spmv(8, 64)

    # the level-3 Laplace solve to 1e-12 against the exact solution
    lap3 = None if args.no_laplace3 else run_laplace_l3()
    # the element-loop Jacobian quadrature on an ensemble's fields
    jq = None if args.no_spmv else run_jac_quad()

    # serving trace (the first --bench-serve-requests requests of the 10,000-request trace)
    served = None
    if not args.no_serve and args.bench_serve_requests > 0:
        nreq = args.bench_serve_requests
        served = {"trace": f"{'all' if nreq >= 10000 else 'the first %d of' % nreq} 10,000 requests, Poisson "
                           f"arrivals at {args.serve_rate:g}/s, levels 3..7, 60% Laplace solves to 1e-10, 40% 10-step "
                           "barvortex integrations, HBM budget 150 GB, lanes opened before the trace",
                  "trace_short": f"{'full' if nreq >= 10000 else 'first %d of' % nreq} 10,000-request trace, "
                                 f"{args.serve_rate:g}/s Poisson, levels 3..7, 60/40 solve/10-step"}
        for name in ("mixed", "fp64"):
            served[name] = run_serve(name, args.bench_serve_requests, args.serve_rate)

    # max over ranks: whole-job rates = every rank's units / the slowest rank's time
    keys = sorted(batched)
    mx = replicas.max_over_ranks([results["mixed"]["ms_per_step"], results["fp64"]["ms_per_step"],
                                  results["mixed"]["e2e_s"]]
                                 + [batched[k][p]["ms_per_step"] for k in keys for p in ("mixed", "fp64")], dev)
    ms, ms64, e2e = mx[:3]
    for i, k in enumerate(keys):
        for j, p in enumerate(("mixed", "fp64")):
            bms = mx[3 + 2 * i + j]
            batched[k][p]["ms_per_step_max_over_ranks"] = bms
            batched[k][p]["member_steps_per_s"] = replicas.whole_job_rate(batched[k]["members"], bms * 1e-3, ws)
        batched[k]["mixed_over_fp64"] = batched[k]["mixed"]["member_steps_per_s"] / batched[k]["fp64"]["member_steps_per_s"]
    if rank != 0:
        replicas.finish()
        return None

    mixed, fp64 = results["mixed"], results["fp64"]
    prof = mixed["prof"]
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = prof["bytes"] / (prof["ms"] * 1e-3) / 1e9 if prof["ms"] > 0 else 0.0
    traffic = None
    tf = os.path.join(HERE, "profiles", "gmres_traffic.json")
    if os.path.exists(tf):
        try:
            traffic = json.load(open(tf)).get("bytes_per_launch")
        except (OSError, ValueError):
            traffic = None
    rel = float(np.linalg.norm(mixed["state"] - fp64["state"]) / np.linalg.norm(fp64["state"]))
    cpu = None
    if ws == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args.level, steps=1, tol=args.tol)
        if lap3 is not None:   # the level-3 solve's error against the CPU reference algorithm's own solve
            ref = cpu.pop("laplace_l3_solution")
            lap3["rel_err_vs_cpu_reference_solve"] = float(np.linalg.norm(lap3.pop("solution") - ref)
                                                           / np.linalg.norm(ref))
        else:
            cpu.pop("laplace_l3_solution", None)
    if lap3 is not None:
        lap3.pop("solution", None)
    def r3(x):
        return None if x is None else float(f"{x:.4g}")

    roof = {"kernel": "gmres_kernel<float>", "bound": "hbm", "achieved": r3(achieved), "peak": peak, "unit": "GB/s",
            "frac": r3(achieved / peak), "traffic": traffic,
            "bytes_per_launch": r3(prof["bytes"] / max(prof["launches"], 1)),
            "ms_per_launch": r3(prof["ms"] / max(prof["launches"], 1)),
            "share_of_step": r3(prof["ms"] / (mixed["eager_ms"] * args.steps)),
            "peak_source": "of measured (MEASURED_PEAKS.json)" if peaks else "of fallback"}
    line = {
        "metric": METRIC,
        "value": ws * 1000.0 / ms,
        "unit": "steps/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64",
        "data": "synthetic (seeded Rossby-Haurwitz wave 4 + spherical-harmonic noise)",
        "config": {"workload": workload(args.level)},
        "solve_tol": args.tol, "parallelism": f"replicas x{ws}", "l2": "flushed between steps (256 MB write)",
        "fp64": {"value": r3(ws * 1000.0 / ms64), "mixed_over_fp64": r3(ms64 / ms)},
        "at_tol_1e-12": None if strict is None else {
            "mixed": r3(strict["mixed"]["steps_per_s"]), "fp64": r3(strict["fp64"]["steps_per_s"])},
        "state_rel_diff_mixed_vs_fp64": r3(rel),
        "batched": {k: {"mixed": r3(v["mixed"]["member_steps_per_s"]), "fp64": r3(v["fp64"]["member_steps_per_s"]),
                        "mixed_over_fp64": r3(v["mixed_over_fp64"]), "rel_err_vs_fp64": r3(v["rel_err_vs_fp64"]),
                        "unit": "member-steps/s"} for k, v in batched.items()} or None,
        "serve": None if served is None else {
            "requests": served["mixed"]["requests"], "trace": served["trace_short"],
            **{p: {"p50_ms": r3(served[p]["p50_ms"]), "p99_ms": r3(served[p]["p99_ms"]),
                   "req_per_s": r3(served[p]["requests_per_s"]), "errors": served[p]["errors"]}
               for p in ("mixed", "fp64")}},
        "spmv": None if spmv is None else {
            "level": spmv["level"], "fp32_x64_frac_of_hbm": r3(spmv["fp32_multivector"]["frac_of_peak"]),
            "fp64_frac_of_hbm": r3(spmv["fp64_single"]["frac_of_peak"])},
        "baroclin": None if baroclin is None else {
            "mixed": r3(baroclin["mixed"]["steps_per_s"]), "fp64": r3(baroclin["fp64"]["steps_per_s"]),
            "mixed_over_fp64": r3(baroclin["mixed_over_fp64"]),
            "rel_diff": r3(baroclin[f"state_rel_diff_mixed_vs_fp64_after_{baroclin['steps']}"])},
        "laplace_l3": None if lap3 is None else {k: (r3(v) if isinstance(v, float) else v) for k, v in lap3.items()},
        "jac_quad": None if jq is None else {"level": jq["level"], "members": jq["members"],
                                            "us_per_call": r3(jq["us_per_call"]),
                                            "frac_of_hbm": r3(jq["frac_of_hbm"])},
        "worst_solve_relres": r3(max(mixed["stats"]["worst_relres"], fp64["stats"]["worst_relres"])),
        "roofline": roof,
        "e2e": {"value": replicas.whole_job_rate(args.steps, e2e, ws), "unit": "steps/s",
                "h2d_bytes_per_step": 8 * (V + 2 * max(os_, 1)), "d2h_bytes_per_step": 8 * V},
        "gpu_launches": mixed["launches"],
        "clocks": mixed["clocks"],
        "cpu_baseline": cpu,
    }
    # everything else (per-path timings, per-level serving, tuned shapes) goes to a side file
    detail = {"fp64": {"ms_per_step": ms64, "path": fp64["path"], "eager_ms": fp64["eager_ms"],
                       "graph_ms": fp64["graph_ms"]},
              "step_path": {"mixed": mixed["path"], "eager_ms": mixed["eager_ms"], "graph_ms": mixed["graph_ms"],
                            "e2e_eager_s": mixed["e2e_eager_s"], "e2e_graph_s": mixed["e2e_graph_s"]},
              "batched": batched, "serve": served, "spmv": spmv, "baroclin": baroclin, "strict": strict,
              "solver": {"mixed": mixed["stats"], "fp64": fp64["stats"]}, "autotuned": tuned or None,
              "roofline_all_solver_launches": {
                  "launches": mixed["prof_all"]["launches"],
                  "share_of_step": mixed["prof_all"]["ms"] / (mixed["eager_ms"] * args.steps),
                  "gbs": mixed["prof_all"]["bytes"] / (mixed["prof_all"]["ms"] * 1e-3) / 1e9
                  if mixed["prof_all"]["ms"] > 0 else None}}
    try:
        os.makedirs(os.path.join(HERE, "gpurun_out"), exist_ok=True)
        with open(os.path.join(HERE, "gpurun_out", "bench_detail.json"), "w") as f:
            json.dump(detail, f, indent=1, default=float)
    except OSError:
        pass
    print(json.dumps(line))
    replicas.finish()
    return line


def workload(level: int) -> str:
    """The timed workload, named by its sizes (a level-L icosahedral sphere has
    10 * 4^L + 2 points and 20 * 4^L triangles); both arms report the same one."""
    return (f"barvortex step, icosahedral level {level} ({10 * 4 ** level + 2} points, {20 * 4 ** level} triangles), "
            "tau=1e-3, theta=0.5, 3 Picard iterations")


def host_threads() -> int:
    """Threads the oracle's OpenMP loops use (OMP_NUM_THREADS, else every host core)."""
    try:
        return max(1, int(os.environ.get("OMP_NUM_THREADS", "")))
    except ValueError:
        return os.cpu_count() or 1


THREAD_NOTE = ("OpenMP over the host cores in the port's parallel loops (assembly, Jacobian right-hand sides, "
               "per-row operator applies); its GMRES+ILU(0) solves are sequential code")


def cpu_baseline(level, steps=1, tol=TOL):
    """The oracle (C restatement of the reference algorithm) on the host:
    timed steps of the bench workload, and (untimed) the level-3 Laplace
    solve of the accuracy leg, the CPU reference answer it is compared with."""
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import pyoracle as po
    from mke_gb300 import fields
    o3 = po.Oracle(3)
    uv3 = o3.mesh_arrays()["uv"].reshape(-1, 4, 2)
    ustar, f = fields.laplace_problem(uv3[:, 0, 0], uv3[:, 0, 1], seed=SEED)
    ref3 = o3.laplace_solve(f, ustar[o3.mesh_arrays()["bnd"] == 1])
    po.set_solver(rel_tol=tol)   # the timed steps: every solve to the GPU arm's tolerance
    o = po.Oracle(level)
    uv = o.mesh_arrays()["uv"].reshape(-1, 4, 2)
    lat, lon = uv[:, 0, 0], uv[:, 0, 1]
    psi, _ = fields.barvortex_initial(lat, lon, seed=SEED)
    bv = o.barvortex(max_iter=3, coriolis=np.sin(lat), **{k: CONF[k] for k in ("tau", "sigma", "mu", "k1", "k2", "theta")})
    z = np.zeros(o.os)
    t0 = time.perf_counter()
    s = psi
    for _ in range(steps):
        s = o.bv_step(bv, s, z, z)
    dt = time.perf_counter() - t0
    return {"value": steps / dt, "unit": "steps/s", "cores": host_threads(), "kind": "port",
            "sample": f"{steps} step(s) of the level-{level} workload after setup; OpenMP loops, sequential "
                      f"GMRES+ILU(0) solves to {tol:g}",
            "laplace_l3_solution": ref3}


def run_reference(args, ws, rank):
    if rank != 0:
        return
    steps = max(1, args.steps)   # about 7 s a step at level 6 on 16 Arm cores: 20 steps ~2.5 min
    warm = min(args.warmup, 1)
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import pyoracle as po
    from mke_gb300 import fields
    po.build()
    po.set_solver(rel_tol=args.tol)   # every solve to the GPU arm's tolerance
    o = po.Oracle(args.level)
    uv = o.mesh_arrays()["uv"].reshape(-1, 4, 2)
    lat, lon = uv[:, 0, 0], uv[:, 0, 1]
    psi, _ = fields.barvortex_initial(lat, lon, seed=SEED)
    bv = o.barvortex(max_iter=3, coriolis=np.sin(lat), **{k: CONF[k] for k in ("tau", "sigma", "mu", "k1", "k2", "theta")})
    z = np.zeros(o.os)
    s = psi
    for _ in range(warm):
        s = o.bv_step(bv, s, z, z)
    t0 = time.perf_counter()
    for _ in range(steps):
        s = o.bv_step(bv, s, z, z)
    dt = time.perf_counter() - t0
    v = steps / dt
    sample = (f"{steps} timed step(s) after {warm} warm-up, level {args.level}, solves to {args.tol:g}; "
              + THREAD_NOTE)
    print(json.dumps({
        "impl": "reference",
        "metric": METRIC,
        "value": v, "unit": "steps/s", "n_gpus": ws, "steps": steps, "warmup": warm,
        "ms_per_step": 1000.0 / v, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded Rossby-Haurwitz wave 4 + spherical-harmonic noise)",
        "config": {"workload": workload(args.level)},
        "cpu_baseline": {"value": v, "unit": "steps/s", "cores": host_threads(), "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def run_jac_quad(level: int = 6, nv: int = 32, reps: int = 20):
    """The element-loop Jacobian quadrature (split pass + k_jac_quad) on the
    fields of an ensemble step: level 6, 32 members, timed with CUDA events on
    its stream, L2 flushed before each call.  Algorithmic bytes: the split
    pass reads both FP64 fields and writes their float pairs (32 V bytes per
    member); the quadrature reads per row its ring (6 x 12 bytes) and the
    row point's cos/sin (8), per member both fields as float pairs (16 V)
    and writes the 8 FP64 right-hand sides (64 rows)."""
    import torch
    from mke_gb300 import fields, phelm
    m = phelm.Mesh.sphere(level)
    lat, lon = m.latlon()
    ops = phelm.Operators(m, phelm.PHG_MIXED)
    J = phelm.SphereJacobian(ops)
    rng = np.random.default_rng(SEED)
    U = np.stack([fields.sh_field(fields.random_coeffs(rng, 1, 12), lat, lon) for _ in range(nv)])
    du = torch.tensor(U, device="cuda")
    dw = torch.roll(du, 1, dims=1).contiguous()
    out = torch.empty((nv, 8, m.inner_size), dtype=torch.float64, device="cuda")
    st = torch.cuda.Stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    with torch.cuda.stream(st):
        J.derivs(du, dw, out, quad=True, stream=st)
        for a, b in ev:
            flush.zero_()
            a.record(st)
            J.derivs(du, dw, out, quad=True, stream=st)
            b.record(st)
    st.synchronize()
    us = sum(a.elapsed_time(b) for a, b in ev) / reps * 1e3
    V, rs = m.size, m.inner_size
    byts = nv * 2 * V * 16 + rs * (6 * 12 + 8) + nv * (2 * V * 8 + 8 * rs * 8)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    return {"level": level, "members": nv, "us_per_call": us, "bytes": byts, "gbs": byts / us / 1e3,
            "frac_of_hbm": byts / us / 1e3 / peak}


def run_laplace_l3(reps: int = 20):
    """The Laplace solve on the level-3 sphere (642 points), GMRES(30) to 1e-12.
    u* = sum of c_lm Y_lm (l = 1..6, c ~ N(0, 1), seeded; l = 0 dropped, so the
    mean is removed), f = Laplacian of u* (exact: -l(l+1) per degree), the
    boundary (south pole) value u*(pole).  FP64 handle, FGMRES(30) to a 1e-12
    relative residual.  Reports iterations, the final residual, the error
    against u* (the discretisation error, O(h^2)) and the solve time."""
    import torch
    from mke_gb300 import fields, phelm
    m = phelm.Mesh.sphere(3)
    lat, lon = m.latlon()
    ustar, f = fields.laplace_problem(lat, lon, seed=SEED)
    bnd = ustar[m.arrays()["bnd"] == 1].copy()
    ops = phelm.Operators(m, phelm.PHG_FP64, restart=30, tol=1e-12)
    L = phelm.SphereLaplace(ops)
    x = L.solve(f, bnd)
    st = ops.last_solve()
    dev = torch.device("cuda")
    df, db = torch.tensor(f, device=dev), torch.tensor(bnd, device=dev)
    out = torch.empty_like(df)
    s = torch.cuda.Stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(s):
        L.solve(df, db, out=out, stream=s)
        e0.record(s)
        for _ in range(reps):
            L.solve(df, db, out=out, stream=s)
        e1.record(s)
    s.synchronize()
    ops.check(s)
    return {"level": 3, "points": m.size, "iters": st["iters"], "relres": st["relres"],
            "rel_err_vs_exact": float(np.linalg.norm(x - ustar) / np.linalg.norm(ustar)),
            "ms_per_solve": e0.elapsed_time(e1) / reps, "solution": x}


def run_serve(precision: str, n: int, rate: float, levels=(3, 4, 5, 6, 7)):
    """The serving trace: n requests with Poisson arrivals at `rate`/s, levels
    uniform over `levels`, 60% Laplace solves to 1e-10 (RHS l <= 10), 40%
    10-step barotropic integrations (RH4 + noise), HBM budget 150 GB.  Lanes
    are opened before the trace (cold start reported separately)."""
    from mke_gb300 import phelm, serve
    prec = phelm.PHG_MIXED if precision == "mixed" else phelm.PHG_FP64
    trace = serve.make_trace(n=n, rate=rate, levels=levels, seed=SEED)
    pools = serve.make_pools(trace, seed=SEED)
    srv = phelm.Server(precision=prec, hbm_budget_bytes=150e9, max_slots=64, solve_tol=1e-10, step_tol=TOL,
                       **CONF)
    t0 = time.perf_counter()
    for kind, level in sorted(pools):
        srv.preload(kind, level)
    cold = time.perf_counter() - t0
    stats, _ = serve.run_trace(srv, trace, pools)
    stats["cold_start_s"] = cold
    stats["bytes_in_use"] = srv.stats()["bytes_in_use"]
    stats["precision"] = precision
    srv.close()
    return stats


def run_spmv(level: int = 8, nv: int = 64, reps: int = 20):
    """Operator apply (phelm::Solver::mult_vector) at a streaming size: the
    Laplacian of a level-`level` mesh applied to nv FP32 vectors (the mixed
    path's SpMV, interleaved members) and to one FP64 vector; L2 flushed
    before every launch, CUDA events around each launch on its stream.
    Algorithmic bytes: the matrix once (column + value per nonzero) plus every
    vector read and written once."""
    import torch
    from mke_gb300 import phelm
    saved = {k: os.environ.get(k) for k in ("PHG_MG", "PHG_CHEB")}
    os.environ["PHG_MG"] = "0"      # no solves here: skip the multigrid setup
    os.environ["PHG_CHEB"] = "0"
    try:
        m = phelm.Mesh.sphere(level)
        ops = phelm.Operators(m, phelm.PHG_MIXED)
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    rs = m.inner_size
    ptr, _, _ = m.csr("lapl")
    nnz = int(ptr[-1])
    dev = torch.device("cuda")
    st = torch.cuda.Stream()
    # flush: write 256 MB (> L2), then read another 256 MB so that the write-backs
    # of the dirty lines happen here and not inside the timed launch
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    clean = torch.zeros(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    g = torch.Generator(device=dev).manual_seed(SEED)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)

    def timed(fn):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        with torch.cuda.stream(st):
            fn()
            for a, b in ev:
                flush.zero_()
                clean.sum()
                a.record(st)
                fn()
                b.record(st)
        st.synchronize()
        return sum(a.elapsed_time(b) for a, b in ev) / reps * 1e3   # us

    x32 = torch.randn(rs, nv, dtype=torch.float32, device=dev, generator=g)   # interleaved members
    y32 = torch.empty_like(x32)
    us32 = timed(lambda: ops.mult32("lapl", x32, y32, stream=st))
    b32 = nnz * 8 + nv * rs * 8
    x64 = torch.randn(rs, dtype=torch.float64, device=dev, generator=g)
    y64 = torch.empty_like(x64)
    us64 = timed(lambda: ops.mult("lapl", x64, out=y64, stream=st))
    b64 = nnz * 12 + rs * 16
    return {"level": level, "rows": rs, "nnz": nnz,
            "l2": "flushed before every launch (256 MB written, then 256 MB of another buffer read)",
            "fp32_multivector": {"members": nv, "layout": "interleaved (rs x nv)", "us_per_launch": us32,
                                 "bytes": b32, "gbs": b32 / us32 / 1e3, "frac_of_peak": b32 / us32 / 1e3 / peak},
            "fp64_single": {"us_per_launch": us64, "bytes": b64, "gbs": b64 / us64 / 1e3,
                            "frac_of_peak": b64 / us64 / 1e3 / peak,
                            "fp64_gops_nonfused": 2.0 * nnz / us64 / 1e3},
            "peak_gbs": peak, "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback"}


BC_CONF = dict(tau=1e-3, sigma=0.05, mu=6.77e-5, sigma1=0.05, mu1=6.77e-5, alpha=0.1 ** 0.5,
               picard_iters=20, picard_tol=1e-8)


def baroclin_initial(lat, lon, seed=SEED):
    """Stream functions of two independent seeded vorticity fields (l <= 12, amplitude 0.05)."""
    from mke_gb300 import fields
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(2):
        c = fields.random_coeffs(rng, 1, 12, 0.05)
        out.append(fields.sh_field(fields.sh_inverse_laplacian(c), lat, lon))
    return out


def run_baroclin(level: int = 6, steps: int = 20, warmup: int = 2):
    """Two-layer baroclinic steps (alpha^2 = 0.1, sigma = 0.05, mu = 6.77e-5,
    sigma1 = sigma, mu1 = mu, tau = 1e-3, Picard up to 20 iterations / 1e-8 as
    in the reference, GMRES(40)), FP64 and mixed; device buffers, events per
    step on the launching stream, L2 flushed between steps."""
    import torch
    from mke_gb300 import phelm
    m = phelm.Mesh.sphere(level)
    lat, lon = m.latlon()
    u1h, u2h = baroclin_initial(lat, lon)
    dev = torch.device("cuda")
    st = torch.cuda.Stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    res = {}
    for name, prec in (("mixed", phelm.PHG_MIXED), ("fp64", phelm.PHG_FP64)):
        ops = phelm.Operators(m, prec, restart=40, tol=TOL)
        bc = phelm.Baroclin(ops, coriolis=np.sin(lat), **BC_CONF)
        u1 = torch.tensor(u1h, device=dev)
        u2 = torch.tensor(u2h, device=dev)
        with torch.cuda.stream(st):
            for _ in range(warmup):
                bc.calc(u1, u2, out1=u1, out2=u2, stream=st)
        st.synchronize()
        u1 = torch.tensor(u1h, device=dev)
        u2 = torch.tensor(u2h, device=dev)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        with torch.cuda.stream(st):
            for a, b in ev:
                flush.zero_()
                a.record(st)
                bc.calc(u1, u2, out1=u1, out2=u2, stream=st)
                b.record(st)
        st.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in ev) / steps
        res[name] = {"steps_per_s": 1000.0 / ms, "ms_per_step": ms, "state": (u1.cpu().numpy(), u2.cpu().numpy())}
        del bc, ops
    (a1, a2), (b1, b2) = res["mixed"].pop("state"), res["fp64"].pop("state")
    diff = max(float(np.linalg.norm(a1 - b1) / np.linalg.norm(b1)), float(np.linalg.norm(a2 - b2) / np.linalg.norm(b2)))
    return {"level": level, "steps": steps, "unknowns": 4 * m.inner_size, "mixed": res["mixed"], "fp64": res["fp64"],
            "mixed_over_fp64": res["mixed"]["steps_per_s"] / res["fp64"]["steps_per_s"],
            f"state_rel_diff_mixed_vs_fp64_after_{steps}": diff,
            "config": "alpha^2=0.1, sigma=sigma1=0.05, mu=mu1=6.77e-5, tau=1e-3, Picard <= 20 / 1e-8, GMRES(40), "
                      "u1, u2 from seeded vorticity l <= 12 amplitude 0.05"}


def run_case(args):
    """Small fixed workloads for profilers: `solve` = Laplace solves,
    `step` = barvortex steps, at --level with --steps repetitions."""
    if args.case == "serve":
        print(json.dumps(run_serve(args.precision, args.serve_requests, args.serve_rate)))
        return
    if args.case == "spmv":
        print(json.dumps(run_spmv(args.level, args.members)))
        return
    if args.case == "baroclin":
        print(json.dumps(run_baroclin(args.level, args.steps)))
        return
    import torch
    from mke_gb300 import phelm
    mesh = phelm.Mesh.sphere(args.level)
    psi0, cor = initial_state(mesh)
    prec = phelm.PHG_MIXED if args.precision == "mixed" else phelm.PHG_FP64
    ops = phelm.Operators(mesh, prec, restart=30, tol=args.tol)
    tune_report = None
    if args.tune:
        tune_report = tune_in_child(args.level, args.precision, args.members if args.case == "batch" else 1)
    u = torch.tensor(psi0, dtype=torch.float64, device="cuda")
    out = torch.empty_like(u)
    zb = torch.zeros(max(mesh.outer_size, 1), dtype=torch.float64, device="cuda")
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    st = torch.cuda.Stream()   # an explicit stream: the library and the events share it
    if args.case == "batch":
        from mke_gb300 import fields
        lat, lon = mesh.latlon()
        B = args.members
        states = np.stack([fields.barvortex_initial(lat, lon, seed=SEED + k, lmax_noise=16)[0] for k in range(B)])
        U = torch.tensor(states, dtype=torch.float64, device="cuda")
        zbB = torch.zeros((B, max(mesh.outer_size, 1)), dtype=torch.float64, device="cuda")
        bv = phelm.BarVortex(ops, coriolis=cor, **CONF)
        bv.calc_batch(U, zbB, zbB, out=U, stream=st)
        if args.graph:
            bv.run(U, 2, zbB, zbB, stream=st)
        torch.cuda.synchronize()
        ev[0].record(st)
        if args.graph:
            bv.run(U, args.steps, zbB, zbB, stream=st)
        else:
            for _ in range(args.steps):
                bv.calc_batch(U, zbB, zbB, out=U, stream=st)
        ev[1].record(st)
        torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[1]) / args.steps
        print(json.dumps({"case": "batch", "level": args.level, "members": B, "precision": args.precision,
                          "ms_per_step": ms, "member_steps_per_s": B * 1000.0 / ms, "graph": args.graph,
                          "tuned": tune_report, "stats": bv.last_stats()}))
        return
    if args.case == "solve":
        L = phelm.SphereLaplace(ops)
        L.solve(u, zb, out=out, stream=st)
        torch.cuda.synchronize()
        ev[0].record(st)
        for _ in range(args.steps):
            L.solve(u, zb, out=out, stream=st)
        ev[1].record(st)
    else:
        bv = phelm.BarVortex(ops, coriolis=cor, **CONF)
        bv.calc(u, zb, zb, out=u, stream=st)
        if args.graph:
            bv.run(u, 2, zb, zb, stream=st)
        torch.cuda.synchronize()
        ev[0].record(st)
        if args.graph:
            bv.run(u, args.steps, zb, zb, stream=st)
        else:
            for _ in range(args.steps):
                bv.calc(u, zb, zb, out=u, stream=st)
        ev[1].record(st)
    torch.cuda.synchronize()
    print(json.dumps({"case": args.case, "level": args.level, "steps": args.steps, "precision": args.precision,
                      "ms_each": ev[0].elapsed_time(ev[1]) / args.steps, "graph": args.graph, "tuned": tune_report,
                      "env": {k: v for k, v in os.environ.items() if k.startswith("PHG_")}}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--level", type=int, default=LEVEL)
    ap.add_argument("--tol", type=float, default=TOL)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-ensemble measurements")
    ap.add_argument("--case", choices=["solve", "step", "batch", "serve", "spmv", "baroclin"],
                    help="one workload only (no bench line): profiling cases, or the serving trace")
    ap.add_argument("--serve-requests", type=int, default=10000, help="requests of --case serve")
    ap.add_argument("--bench-serve-requests", type=int, default=2000, help="requests of the bench line's serve block")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving trace")
    ap.add_argument("--no-spmv", action="store_true", help="skip the streaming operator-apply measurement")
    ap.add_argument("--no-baroclin", action="store_true", help="skip the two-layer baroclinic steps")
    ap.add_argument("--no-laplace3", action="store_true", help="skip the level-3 Laplace solve accuracy leg")
    ap.add_argument("--serve-rate", type=float, default=2000.0)
    ap.add_argument("--members", type=int, default=16, help="ensemble members for --case batch")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--graph", action="store_true", help="--case step / batch: replay one captured step")
    ap.add_argument("--tune", action="store_true", help="--case step / batch: autotune the launch shapes first")
    ap.add_argument("--no-tune", action="store_true", help="bench line: keep the default launch shapes")
    args = ap.parse_args()
    if args.case:
        run_case(args)
        return
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    if args.warmup < 3:
        args.warmup = 3
    run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()
