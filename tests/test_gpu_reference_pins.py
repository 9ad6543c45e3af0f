"""The reference's own accuracy checks, run on the GPU path.

* Sphere Laplacian (examples/test_slaplace.cpp:100-199, thresholds
  scripts/test_slaplace.lua:25-54): solve Laplacian(u) = f with the pole
  value of u as boundary condition ("L1: invert", error e1 against u), apply
  the Laplacian to u ("L2"), solve again from that result ("L3", the round
  trip, <= 1e-7); e1 must fall by >= 3.3 from level 3 to 4 and from 4 to 5.
* Barotropic vorticity with a manufactured solution
  (examples/test_barvortex.cpp:216-242, 488-559, thresholds
  scripts/test_barvortex.lua:28-42): psi = phi cos^4(phi) sin(lam + t), no
  Coriolis term, the forcing that makes psi exact, tau = 1e-3 up to T = 0.01;
  the SphereNorm distance to psi(T) must fall by >= 2 from level 4 to 5.
* Spherical Jacobian of an analytic pair (examples/test_barvortex.cpp:57-105,
  scripts/test_jacobian.lua:28-33).

The reference's own figures on these inputs (tests/golden/ref_pins.npz, its
sources run by tests/golden/make_golden.py) are the pins: each error here
must equal the reference's.  On the full-sphere mesh (south pole as the only
boundary point) the reference does not meet two of its script thresholds
itself: the manufactured barotropic error is 1.2e-3 at level 4 and 1.1e-4 at
level 5 (thresholds 1e-4 and 1e-5; the ratio, 11, passes), and the analytic
Jacobian's exact value is singular at the north pole, an inner point of this
mesh (1/cos(pi/2)), so the distance is 8.1e14 (threshold 1).  Those two are
checked against the reference's figures and the ratio only.

Errors are SphereNorm distances (src/norm.h:81-105), as the reference prints
them.  Both precisions must pass; the mixed path's solves are refined to the
same FP64 residual.
"""
import numpy as np
import pytest

import manufactured as mf
from mke_gb300 import phelm

pytestmark = pytest.mark.gpu

PRECISIONS = [phelm.PHG_FP64, phelm.PHG_MIXED]


def chart(m):
    lat, lon = m.latlon()
    return lat, lon, m.arrays()["bnd"] == 1


def slaplace_errors(level, precision):
    m = phelm.Mesh.sphere(level)
    lat, lon, isb = chart(m)
    ops = phelm.Operators(m, precision, tol=1e-12)
    L, N = phelm.SphereLaplace(ops), phelm.SphereNorm(ops)
    u = mf.slaplace_u(lat, lon)
    lu = mf.slaplace_lapl(lat, lon)
    inv = L.solve(lu, u[isb])                   # "L1: invert"
    e1 = N.dist(inv, u)
    lu1 = L.calc1(u, lu[isb])                   # "L2: laplace"
    e2 = N.dist(lu, lu1)
    back = L.solve(lu1, u[isb])                 # "L3": the round trip
    e3 = N.dist(u, back)
    return e1, e2, e3


@pytest.mark.parametrize("precision", PRECISIONS)
def test_slaplace_convergence_and_round_trip(precision, golden):
    ref = golden("ref_pins.npz")
    e = {lv: slaplace_errors(lv, precision) for lv in (3, 4, 5)}
    for lv, (e1, e2, e3) in e.items():
        r1, r2, _ = ref[f"slaplace_L{lv}"]
        assert e3 <= 1e-7, (lv, e3)                     # the round trip
        # the reference's own errors: equal up to the solves' tolerance (a 1e-12
        # residual moves a level-5 solution by up to ~1e-7 of its norm)
        assert abs(e1 - r1) <= 1e-6 * r1, (lv, e1, r1)
        assert abs(e2 - r2) <= 1e-8 * r2, (lv, e2, r2)
    assert e[3][0] / e[4][0] >= 3.3, e
    assert e[4][0] / e[5][0] >= 3.3, e


def barvortex_error(level, precision):
    m = phelm.Mesh.sphere(level)
    lat, lon, isb = chart(m)
    ops = phelm.Operators(m, precision, tol=1e-12)
    tau, sigma, mu, T = 1e-3, 1.6e-2, 8e-5, 0.01
    # no Coriolis term; Picard iterations up to the reference's 1e-14 stop test
    bv = phelm.BarVortex(ops, tau=tau, sigma=sigma, mu=mu, k1=1.0, k2=1.0, theta=0.5, picard_iters=100,
                         coriolis=np.zeros(m.size))
    N = phelm.SphereNorm(ops)
    u = mf.bv_psi(lat, lon, 0.0)
    zb = np.zeros(m.outer_size)
    t = 0.0
    while t < T:            # the reference's loop: t accumulates tau (11 steps to T = 0.01)
        u = bv.calc(u, zb, zb, forcing=mf.bv_forcing(lat, lon, t, sigma, mu))
        t += tau
    return N.dist(u, mf.bv_psi(lat, lon, t))


@pytest.mark.parametrize("precision", PRECISIONS)
def test_barvortex_manufactured_solution(precision, golden):
    ref = golden("ref_pins.npz")
    e4 = barvortex_error(4, precision)
    e5 = barvortex_error(5, precision)
    assert abs(e4 - ref["barvortex_L4"][0]) <= 1e-6 * e4, (e4, ref["barvortex_L4"])
    assert abs(e5 - ref["barvortex_L5"][0]) <= 1e-6 * e5, (e5, ref["barvortex_L5"])
    assert e4 / e5 >= 2.0, (e4, e5)


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("level", [3, 4, 5])
def test_jacobian_analytic(precision, level, golden):
    import pyoracle as po
    ref = golden("ref_pins.npz")
    m = phelm.Mesh.sphere(level)
    lat, lon, isb = chart(m)
    ops = phelm.Operators(m, precision, tol=1e-12)
    J, N = phelm.SphereJacobian(ops), phelm.SphereNorm(ops)
    exact = mf.jac_exact(lat, lon)
    f1, f2 = mf.jac_f1(lat, lon), mf.jac_f2(lat, lon)
    got = J.calc1(f1, f2, exact[isb])
    r = ref[f"jacobian_L{level}"][0]
    assert abs(N.dist(got, exact) - r) <= 1e-9 * r
    # the values themselves, against the oracle (the reference's arithmetic)
    want = po.Oracle(level).jacobian_calc1(f1, f2, exact[isb])
    inner = ~isb      # the boundary value is the (singular) input itself
    assert np.linalg.norm(got[inner] - want[inner]) <= 1e-13 * np.linalg.norm(want[inner])
