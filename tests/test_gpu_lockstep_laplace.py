"""Lockstep multigrid FGMRES for many Laplace right-hand sides at once (the
mixed path's ensemble Laplace solves).  Forced through the launch-shape table
(family 2 = multigrid-preconditioned GMRES, path 1 = lockstep) and compared
with the per-member persistent solver and with single solves.  Both run to a
1e-12 relative residual, so they agree to 1e-9 relative L2 (the tolerance of
the other solve tests)."""
import numpy as np
import pytest

from mke_gb300 import fields, phelm, serve

pytestmark = pytest.mark.gpu

TOL = 1e-9
CONF = dict(tau=1e-3, sigma=1.6e-2, mu=8e-5, theta=0.5, picard_iters=3)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


def force_path(tmp_path, rows, nv, path):
    """A table entry for the multigrid Laplacian of `rows` rows at nv right-hand sides (mixed precision)."""
    head = tmp_path / "h.txt"
    phelm.tune_clear()
    phelm.tune_save(str(head))
    f = tmp_path / "t.txt"
    bucket = (nv - 1).bit_length()
    f.write_text(head.read_text().splitlines()[0] + f"\nsolve 2 {rows} 1 {bucket} 0 {path}\n")
    assert phelm.tune_load(str(f)) == 1


@pytest.fixture(autouse=True)
def clean_table():
    phelm.tune_clear()
    yield
    phelm.tune_clear()


@pytest.mark.parametrize("level,nv", [(3, 8), (4, 32), (5, 13)])
def test_batch_solve_matches_per_member(tmp_path, level, nv):
    m = phelm.Mesh.sphere(level)
    lat, lon = m.latlon()
    F = serve.solve_inputs(lat, lon, nv, seed=100 + level)
    ops = phelm.Operators(m, phelm.PHG_MIXED, tol=1e-12)
    L = phelm.SphereLaplace(ops)
    force_path(tmp_path, m.inner_size, nv, 0)
    per_member = L.solve_batch(F)
    force_path(tmp_path, m.inner_size, nv, 1)
    k0 = phelm.kernel_launches()
    lock = L.solve_batch(F)
    assert phelm.kernel_launches() - k0 > 100      # the lockstep launches ran
    st = ops.last_solve()
    assert st["relres"] <= 1e-12 and st["iters"] > 0
    assert rel(lock, per_member) <= TOL
    # and each member equals its own single solve
    for k in (0, nv - 1):
        assert rel(lock[k], L.solve(F[k])) <= TOL


def test_zero_and_repeated_right_hand_sides(tmp_path):
    m = phelm.Mesh.sphere(4)
    lat, lon = m.latlon()
    F = serve.solve_inputs(lat, lon, 9, seed=5)
    F[3] = 0.0
    F[7] = F[2]
    ops = phelm.Operators(m, phelm.PHG_MIXED, tol=1e-12)
    L = phelm.SphereLaplace(ops)
    force_path(tmp_path, m.inner_size, 9, 1)
    X = L.solve_batch(F)
    assert np.all(np.isfinite(X))
    assert np.array_equal(X[7], X[2])
    force_path(tmp_path, m.inner_size, 9, 0)
    ref = L.solve_batch(F)
    assert rel(X, ref) <= TOL


def test_ensemble_steps_graph_replayed(tmp_path):
    """The barotropic ensemble step with its Laplace solves in lockstep, enqueued
    kernel by kernel and replayed from a captured graph."""
    m = phelm.Mesh.sphere(4)
    lat, lon = m.latlon()
    ops = phelm.Operators(m, phelm.PHG_MIXED, tol=1e-12)
    bv = phelm.BarVortex(ops, coriolis=np.sin(lat), **CONF)
    U0 = np.stack([fields.barvortex_initial(lat, lon, seed=60 + k)[0] for k in range(16)])
    force_path(tmp_path, m.inner_size, 16, 0)
    ref = U0.copy()
    for _ in range(3):
        ref = bv.calc_batch(ref)
    force_path(tmp_path, m.inner_size, 16, 1)
    a = U0.copy()
    for _ in range(3):
        a = bv.calc_batch(a)
    assert rel(a, ref) <= TOL
    b = U0.copy()
    bv.run(b, 3)
    assert np.array_equal(a, b)
    assert bv.last_stats()["worst_relres"] <= 1e-10
