"""Captured steps (phg_barvortex_run): one barotropic step captured as a CUDA
graph and replayed.  The replayed kernels read and write the same buffers in
the same order as the step enqueued kernel by kernel, so K replayed steps
equal K calls of calc / calc_batch bit for bit."""
import numpy as np
import pytest

from mke_gb300 import fields, phelm

pytestmark = pytest.mark.gpu

CONF = dict(tau=1e-3, sigma=1.6e-2, mu=8e-5, theta=0.5, picard_iters=3)


def states(m, n, seed=0):
    lat, lon = m.latlon()
    return np.stack([fields.barvortex_initial(lat, lon, seed=seed + k, lmax_noise=16)[0] for k in range(n)])


@pytest.mark.parametrize("precision", [phelm.PHG_FP64, phelm.PHG_MIXED])
def test_run_equals_step_loop_host(precision):
    m = phelm.Mesh.sphere(4)
    lat, _ = m.latlon()
    ops = phelm.Operators(m, precision, tol=1e-12)
    bv = phelm.BarVortex(ops, coriolis=np.sin(lat), **CONF)
    u0 = states(m, 1)[0]
    ref = u0.copy()
    for _ in range(5):
        ref = bv.calc(ref)
    u = u0.copy()
    bv.run(u, 5)
    assert np.array_equal(u, ref)
    # the graph is kept: 3 more steps replay it, and continue the same trajectory
    for _ in range(3):
        ref = bv.calc(ref)
    k0 = phelm.kernel_launches()
    bv.run(u, 3)
    assert np.array_equal(u, ref)
    per_replay = (phelm.kernel_launches() - k0) / 3
    assert per_replay > 10   # every kernel of a step is counted once per replay
    st = bv.last_stats()
    assert st["worst_relres"] <= 1e-10


def test_run_batch_on_device_stream():
    torch = pytest.importorskip("torch")
    m = phelm.Mesh.sphere(4)
    lat, _ = m.latlon()
    ops = phelm.Operators(m, phelm.PHG_MIXED, tol=1e-12)
    bv = phelm.BarVortex(ops, coriolis=np.sin(lat), **CONF)
    U0 = states(m, 6, seed=40)
    ref = U0.copy()
    for _ in range(4):
        ref = bv.calc_batch(ref)
    s = torch.cuda.Stream()
    U = torch.tensor(U0, device="cuda")
    zb = torch.zeros((6, m.outer_size), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    bv.run(U, 1, zb, zb, stream=s)       # no graph yet: enqueued kernel by kernel
    bv.run(U, 3, zb, zb, stream=s)       # replays
    s.synchronize()
    assert np.array_equal(U.cpu().numpy(), ref)
    assert bv.last_stats()["worst_relres"] <= 1e-10


def test_graph_recaptured_after_reallocation():
    """A larger batch on the same handle reallocates the step buffers; the
    graph captured before must not be replayed with the old addresses."""
    m = phelm.Mesh.sphere(3)
    lat, _ = m.latlon()
    ops = phelm.Operators(m, phelm.PHG_FP64, tol=1e-12)
    bv = phelm.BarVortex(ops, coriolis=np.sin(lat), **CONF)
    u0 = states(m, 1, seed=7)[0]
    u = u0.copy()
    bv.run(u, 3)
    bv.calc_batch(states(m, 16, seed=8))   # grows every step buffer
    bv.run(u, 3)
    ref = u0.copy()
    for _ in range(6):
        ref = bv.calc(ref)
    assert np.array_equal(u, ref)


def test_run_arguments():
    m = phelm.Mesh.sphere(2)
    ops = phelm.Operators(m, phelm.PHG_FP64)
    bv = phelm.BarVortex(ops, **CONF)
    u = states(m, 1)[0]
    v = u.copy()
    bv.run(v, 0)
    assert np.array_equal(u, v)
    with pytest.raises(phelm.PhgError):
        bv.run(v, -1)
