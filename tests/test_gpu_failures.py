"""Failure detection without a GPU fault: invalid inputs and exhausted
iteration budgets end in an error status from the library (every solver loop
is bounded by iteration and cycle caps and a stagnation test, every group
barrier by a time limit), and the handle stays usable afterwards."""
import numpy as np
import pytest

from mke_gb300 import fields, phelm, serve

pytestmark = pytest.mark.gpu

NOT_CONVERGED = 3
CONF = dict(tau=1e-3, sigma=1.6e-2, mu=8e-5, theta=0.5, picard_iters=3)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


@pytest.mark.parametrize("precision", [phelm.PHG_FP64, phelm.PHG_MIXED])
def test_non_finite_right_hand_side(precision):
    m = phelm.Mesh.sphere(4)
    lat, lon = m.latlon()
    ops = phelm.Operators(m, precision, tol=1e-12)
    L = phelm.SphereLaplace(ops)
    F = serve.solve_inputs(lat, lon, 1, seed=3)[0]
    good = L.solve(F)
    bad = F.copy()
    bad[17] = np.nan
    with pytest.raises(phelm.PhgError) as e:
        L.solve(bad)
    assert e.value.code == NOT_CONVERGED
    # the context and the handle are fine
    assert np.array_equal(L.solve(F), good)


def test_non_finite_ensemble_member_lockstep():
    """One NaN member among 16 in the lockstep ensemble solver: the call
    reports it; the handle then solves clean ensembles again."""
    m = phelm.Mesh.sphere(5)
    lat, lon = m.latlon()
    ops = phelm.Operators(m, phelm.PHG_MIXED, tol=1e-12)
    L = phelm.SphereLaplace(ops)
    F = serve.solve_inputs(lat, lon, 16, seed=4)
    good = L.solve_batch(F)
    bad = F.copy()
    bad[5, 100] = np.inf
    with pytest.raises(phelm.PhgError) as e:
        L.solve_batch(bad)
    assert e.value.code == NOT_CONVERGED
    assert rel(L.solve_batch(F), good) <= 1e-12


def test_non_finite_state_in_a_step():
    m = phelm.Mesh.sphere(4)
    lat, lon = m.latlon()
    ops = phelm.Operators(m, phelm.PHG_FP64, tol=1e-12)
    bv = phelm.BarVortex(ops, coriolis=np.sin(lat), **CONF)
    u = fields.barvortex_initial(lat, lon, seed=1)[0]
    good = bv.calc(u)
    bad = u.copy()
    bad[0] = np.nan
    with pytest.raises(phelm.PhgError):
        bv.calc(bad)
    assert np.array_equal(bv.calc(u), good)


def test_iteration_cap():
    m = phelm.Mesh.sphere(5)
    lat, lon = m.latlon()
    ops = phelm.Operators(m, phelm.PHG_FP64, tol=1e-12)
    L = phelm.SphereLaplace(ops)
    F = serve.solve_inputs(lat, lon, 1, seed=8)[0]
    good = L.solve(F)
    ops.set_solver(restart=30, tol=1e-12, max_iter=2)
    with pytest.raises(phelm.PhgError) as e:
        L.solve(F)
    assert e.value.code == NOT_CONVERGED
    assert ops.last_solve()["iters"] <= 2
    ops.set_solver(restart=30, tol=1e-12, max_iter=20000)
    assert rel(L.solve(F), good) <= 1e-9


@pytest.mark.parametrize("precision", [phelm.PHG_FP64, phelm.PHG_MIXED])
@pytest.mark.parametrize("level", [3, 4, 6])
def test_device_index_arrays_in_range(level, precision):
    """phg_ops_validate reads every device index array of a handle (patterns,
    maps, boundary lists, multigrid transfers) and finds none out of range."""
    ops = phelm.Operators(phelm.Mesh.sphere(level), precision)
    assert ops.validate() == 0


TIMEOUT = 4


@pytest.mark.parametrize("precision", [phelm.PHG_FP64, phelm.PHG_MIXED])
def test_barrier_wait_runs_out(precision):
    """A device-side wait made to run out: with a wait limit of one clock
    cycle every group-barrier wait of the persistent multigrid solver (161
    blocks share one level-6 Laplace solve) gives up at once, sets the
    launch's error flag and returns; the call reports PHG_ERR_TIMEOUT.  Back
    at the default limit the same handle solves the same input again."""
    m = phelm.Mesh.sphere(6)
    lat, lon = m.latlon()
    ops = phelm.Operators(m, precision, tol=1e-12)
    L = phelm.SphereLaplace(ops)
    F = serve.solve_inputs(lat, lon, 1, seed=5)[0]
    good = L.solve(F)
    ops.set_wait_limit(1)
    with pytest.raises(phelm.PhgError) as e:
        L.solve(F)
    assert e.value.code == TIMEOUT
    ops.set_wait_limit(0)
    assert rel(L.solve(F), good) <= 1e-9
    assert ops.last_solve()["relres"] <= 1e-12
