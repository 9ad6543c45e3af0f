"""Laplace solves on meshes of different levels in one persistent launch
(phg_laplace_solve_levels): every right-hand side equals the same solve on
its own mesh alone (phg_laplace_solve_batch) to the solve tolerance, against
the oracle too, in both precisions, with boundary values, host and device
arrays."""
import numpy as np
import pytest

import pyoracle as po
from mke_gb300 import phelm, serve

pytestmark = pytest.mark.gpu

LEVELS = (3, 4, 5)


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def problem(level, nv, seed):
    m = phelm.Mesh.sphere(level)
    lat, lon = m.latlon()
    F = serve.solve_inputs(lat, lon, nv, seed=seed)
    bnd = np.stack([F[k][m.arrays()["bnd"] == 1] * 0.5 for k in range(nv)])
    return m, F, bnd


@pytest.mark.parametrize("precision", [phelm.PHG_FP64, phelm.PHG_MIXED])
def test_levels_equal_single_meshes(precision):
    nvs = (3, 2, 4)
    probs = [problem(lv, nv, 30 + lv) for lv, nv in zip(LEVELS, nvs)]
    ops = [phelm.Operators(m, precision, tol=1e-12) for m, _, _ in probs]
    outs = phelm.laplace_solve_levels(ops, [F for _, F, _ in probs], [b for _, _, b in probs])
    assert ops[0].last_solve()["relres"] <= 1e-12
    for (m, F, bnd), o, got in zip(probs, ops, outs):
        want = phelm.SphereLaplace(o).solve_batch(F, bnd)
        for k in range(F.shape[0]):
            assert rel(got[k], want[k]) <= 1e-9, (m.size, k)
    # one member of each mesh against the oracle (the reference's algorithm)
    for (m, F, bnd), got, lv in zip(probs, outs, LEVELS):
        want = po.Oracle(lv).laplace_solve(F[0], bnd[0])
        assert rel(got[0], want) <= 1e-9


def test_levels_device_arrays():
    import torch
    probs = [problem(lv, 2, 50 + lv) for lv in LEVELS]
    ops = [phelm.Operators(m, phelm.PHG_MIXED, tol=1e-12) for m, _, _ in probs]
    Fd = [torch.tensor(F, device="cuda") for _, F, _ in probs]
    s = torch.cuda.Stream()
    outs = phelm.laplace_solve_levels(ops, Fd, stream=s)
    ops[0].check(s)        # device arrays: the call only enqueued the work
    for (m, F, _), o, got in zip(probs, ops, outs):
        want = phelm.SphereLaplace(o).solve_batch(F)
        assert rel(got.cpu().numpy(), want) <= 1e-9


def test_levels_refusals():
    m3 = phelm.Mesh.sphere(3)
    a = phelm.Operators(m3, phelm.PHG_FP64)
    b = phelm.Operators(m3, phelm.PHG_MIXED)
    F = np.zeros((1, m3.size))
    with pytest.raises(phelm.PhgError) as e:
        phelm.laplace_solve_levels([a, b], [F, F])
    assert e.value.code == 1


@pytest.mark.parametrize("sms", [1, 3, 8, 40])
def test_levels_few_sms(sms):
    """The resident blocks split between the meshes in proportion to their
    work, at least one block each (one SM: three blocks for three meshes,
    beyond the cap): with the launch capped to a few SMs the
    small meshes get single-block groups and several right-hand sides per
    group; every solution still equals the mesh's own batched solve."""
    nvs = (5, 3, 2)
    probs = [problem(lv, nv, 60 + lv) for lv, nv in zip(LEVELS, nvs)]
    ops = [phelm.Operators(m, phelm.PHG_MIXED, tol=1e-12) for m, _, _ in probs]
    ops[0].set_sms(sms)
    outs = phelm.laplace_solve_levels(ops, [F for _, F, _ in probs], [b for _, _, b in probs])
    ops[0].set_sms(0)
    for (m, F, bnd), o, got in zip(probs, ops, outs):
        want = phelm.SphereLaplace(o).solve_batch(F, bnd)
        for k in range(F.shape[0]):
            assert rel(got[k], want[k]) <= 1e-9, (sms, m.size, k)
