"""The benchmarked ensemble path at its benchmarked sizes.

Level 5 x 256 members and level 6 x 32 members in mixed precision run as the
bench runs them: the default launch shapes (lockstep Chebyshev mass solves,
lockstep multigrid FGMRES Laplace solves, element-loop Jacobian right-hand
sides) inside one captured and replayed step graph (phg_barvortex_run).
Members are compared with their own single-trajectory FP64 steps and one
member with the oracle (the reference algorithm on the CPU), all through the
C ABI.  Tolerance: 1e-9 relative L2 of the state (every solve is refined to a
1e-12 FP64 residual; the FP32 Jacobian quadrature moves a step by ~1e-11).
"""
import numpy as np
import pytest

import pyoracle as po
from mke_gb300 import fields, phelm

pytestmark = pytest.mark.gpu

SEED = 2024
CONF = dict(tau=1e-3, sigma=1.6e-2, mu=8e-5, k1=1.0, k2=1.0, theta=0.5, picard_iters=3)


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def ensemble(level, members, steps, check, oracle_steps):
    import torch
    m = phelm.Mesh.sphere(level)
    lat, lon = m.latlon()
    states = np.stack([fields.barvortex_initial(lat, lon, seed=SEED + k, lmax_noise=16)[0] for k in range(members)])
    cor = np.sin(lat)
    mixed = phelm.Operators(m, phelm.PHG_MIXED, tol=1e-12)
    bv = phelm.BarVortex(mixed, coriolis=cor, **CONF)
    U = torch.tensor(states, device="cuda")
    zb = torch.zeros((members, max(m.outer_size, 1)), dtype=torch.float64, device="cuda")
    s = torch.cuda.Stream()
    bv.run(U, steps, zb, zb, stream=s)
    s.synchronize()
    st = bv.last_stats()
    assert st["worst_relres"] <= 1e-11, st
    got = U.cpu().numpy()
    fp64 = phelm.Operators(m, phelm.PHG_FP64, tol=1e-12)
    bv64 = phelm.BarVortex(fp64, coriolis=cor, **CONF)
    z = np.zeros(m.outer_size)
    for k in check:
        x = states[k].copy()
        for _ in range(steps):
            x = bv64.calc(x, z, z)
        assert rel(got[k], x) <= 1e-9, (k, rel(got[k], x))
    o = po.Oracle(level)
    obv = o.barvortex(max_iter=3, coriolis=cor)
    x = states[check[0]].copy()
    for _ in range(oracle_steps):
        x = o.bv_step(obv, x, z, z)
    if oracle_steps == steps:
        assert rel(got[check[0]], x) <= 1e-9
    else:   # a shorter oracle run, against the mixed ensemble replayed for as many steps
        U2 = torch.tensor(states, device="cuda")
        bv.run(U2, oracle_steps, zb, zb, stream=s)
        s.synchronize()
        assert rel(U2[check[0]].cpu().numpy(), x) <= 1e-9
    return got


def test_level5_256_members():
    """The ensemble workload: 256 members on level 5, 10 steps;
    members 0, 97 and 255 against their FP64 single trajectories, member 0
    against the oracle."""
    ensemble(5, 256, 10, check=(0, 97, 255), oracle_steps=10)


def test_level6_32_members():
    """32 members on level 6, 5 steps; members 0 and 31 against their FP64
    single trajectories, member 0 against the oracle for 2 steps."""
    ensemble(6, 32, 5, check=(0, 31), oracle_steps=2)
