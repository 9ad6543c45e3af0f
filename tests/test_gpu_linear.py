"""Linearised and adjoint barotropic steps on the GPU against the reference.

BarVortex::calc_L (the step linearised around a background state z),
calc_L_1 (its inverse, with the backward Crank-Nicolson matrix) and calc_LT
(the adjoint), examples/barvortex_impl.h:326-536, around z = in_u applied to
in_v with zero boundaries.  Each solves systems with the A / Ab matrices and
the Laplacian, to 1e-12 relative residual here and 1e-13 in the reference:
1e-9 relative L2, the tolerance of the other solve-based tests.
"""
import numpy as np
import pytest

from mke_gb300 import phelm

pytestmark = pytest.mark.gpu

TOL = 1e-9


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("precision", [phelm.PHG_FP64, phelm.PHG_MIXED])
@pytest.mark.parametrize("level", [1, 2, 3, 4])
def test_linear_steps_vs_reference(golden, level, precision):
    g = golden(f"ref_L{level}.npz")
    m = phelm.Mesh.sphere(level)
    ops = phelm.Operators(m, precision, tol=1e-12)
    lat, _ = m.latlon()
    bv = phelm.BarVortex(ops, tau=1e-3, sigma=1.6e-2, mu=8e-5, k1=1.0, k2=1.0, theta=0.5, picard_iters=3,
                         coriolis=np.sin(lat))
    z = np.zeros(m.outer_size)
    assert rel(bv.calc_L(g["in_v"], g["in_u"], z, z), g["out_bv_L"]) <= TOL
    assert rel(bv.calc_L_1(g["in_v"], g["in_u"], z, z), g["out_bv_L1"]) <= TOL
    assert rel(bv.calc_LT(g["in_v"], g["in_u"], z, z), g["out_bv_LT"]) <= TOL


def test_calc_L_1_accumulates_and_aliases(golden):
    """calc_L_1 adds into its output as the reference does; outputs may alias inputs."""
    torch = pytest.importorskip("torch")
    g = golden("ref_L3.npz")
    m = phelm.Mesh.sphere(3)
    ops = phelm.Operators(m, phelm.PHG_FP64, tol=1e-12)
    lat, _ = m.latlon()
    bv = phelm.BarVortex(ops, picard_iters=3, coriolis=np.sin(lat))
    base = bv.calc_L_1(g["in_v"], g["in_u"])
    acc = np.full(m.size, 0.5)
    got = bv.calc_L_1(g["in_v"], g["in_u"], out=acc.copy())
    want = bv.calc_L_1(g["in_v"], g["in_u"], out=acc.copy())
    assert np.array_equal(got, want)
    assert rel(got, base) > 1e-6          # the start value matters
    s = torch.cuda.Stream()
    u = torch.tensor(g["in_v"], device="cuda")
    zz = torch.tensor(g["in_u"], device="cuda")
    ref = bv.calc_L(g["in_v"], g["in_u"])
    bv.calc_L(u, zz, out=u, stream=s)
    s.synchronize()
    assert rel(u.cpu().numpy(), ref) <= 1e-12


@pytest.mark.parametrize("precision", [phelm.PHG_FP64, phelm.PHG_MIXED])
@pytest.mark.parametrize("level", [1, 2, 3])
def test_baroclin_linear_steps_vs_reference(golden, level, precision):
    """Baroclin::calc_L / calc_L_1 around (z1, z2) = (in_u, in_v) applied to
    (in_v, in_u) (examples/baroclin.cpp:620-986), zero boundary."""
    g = golden(f"ref_L{level}.npz")
    m = phelm.Mesh.sphere(level)
    ops = phelm.Operators(m, precision, tol=1e-12)
    lat, _ = m.latlon()
    bc = phelm.Baroclin(ops, picard_iters=3, coriolis=np.sin(lat))
    z = np.zeros(m.outer_size)
    for which, fn in (("L", bc.calc_L), ("L1", bc.calc_L_1)):
        a, b = fn(g["in_v"], g["in_u"], g["in_u"], g["in_v"], z)
        assert rel(a, g[f"out_bc_{which}_u1"]) <= TOL, which
        assert rel(b, g[f"out_bc_{which}_u2"]) <= TOL, which
