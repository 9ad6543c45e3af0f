"""The V-cycle's cluster tail: the coarse parallel levels run inside the
group's first thread-block cluster (distributed shared memory, hardware
cluster barriers) instead of over the whole group.  It is off by default
(measured slower on the level-6 step) and turned on per handle with
PHG_MG_CLUSTER=8 at operator creation.  Its arithmetic is the group-wide
levels' arithmetic, so with the same group shape a solve with the tail
returns the same bits as one without.  The group shape is pinned with PHG_ROWS_PER_BLOCK so that both
launches split the rows over the same 160 blocks (a multiple of the cluster
size, which the tail needs)."""
import numpy as np
import pytest

from mke_gb300 import fields, phelm, serve

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [phelm.PHG_FP64, phelm.PHG_MIXED])
def test_tail_equals_group_levels(precision, monkeypatch):
    m = phelm.Mesh.sphere(6)
    lat, lon = m.latlon()
    F = serve.solve_inputs(lat, lon, 2, seed=21)
    monkeypatch.setenv("PHG_ROWS_PER_BLOCK", "257")   # ceil(40961 / 257) = 160 blocks either way
    monkeypatch.setenv("PHG_MG_CLUSTER", "8")
    with_tail = phelm.Operators(m, precision, tol=1e-12)
    monkeypatch.setenv("PHG_MG_CLUSTER", "0")
    without = phelm.Operators(m, precision, tol=1e-12)
    monkeypatch.delenv("PHG_MG_CLUSTER")
    for k in range(2):
        a = phelm.SphereLaplace(with_tail).solve(F[k])
        st = with_tail.last_solve()
        b = phelm.SphereLaplace(without).solve(F[k])
        assert st == without.last_solve()
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), k
        assert st["relres"] <= 1e-12


def test_tail_batch(monkeypatch):
    """A batch of Laplace solves (one group per right-hand side, each group
    with its own cluster tail and tail counter) equals the single solves."""
    m = phelm.Mesh.sphere(5)
    lat, lon = m.latlon()
    monkeypatch.setenv("PHG_MG_CLUSTER", "8")
    ops = phelm.Operators(m, phelm.PHG_FP64, tol=1e-12)
    monkeypatch.delenv("PHG_MG_CLUSTER")
    L = phelm.SphereLaplace(ops)
    F = serve.solve_inputs(lat, lon, 3, seed=5)
    B = L.solve_batch(F)
    for k in range(3):
        one = L.solve(F[k])
        assert np.linalg.norm(B[k] - one) <= 1e-10 * np.linalg.norm(one)
