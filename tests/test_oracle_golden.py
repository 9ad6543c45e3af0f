"""The CPU oracle against the reference's own results and known answers.

Pins: tests/golden/ref_L*.npz were produced by the reference's sources
(oracle/_ref, see tests/golden/make_golden.py); the integration known-answer
values come from the reference's unit tests (tests/test_integrate.cpp:41-43,
76-88, 166-270 and tests/test_quadrature.c:31-38 in the reference tree).
"""
import ctypes as C
import math

import numpy as np
import pytest

import pyoracle as po

OPS = ["idt", "lapl", "bnd1", "bnd2", "bnd3", "jidt", "d1", "d2", "d1c", "d2c",
       "d1b", "d2b", "d1cb", "d2cb", "norm"]


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.int64)


@pytest.fixture(scope="module", params=[1, 2, 3])
def lvl(request, golden):
    return request.param, po.Oracle(request.param), golden(f"ref_L{request.param}.npz")


def test_mesh_bitexact(lvl):
    level, o, g = lvl
    ma = o.mesh_arrays()
    for k in ("tri", "tz", "bnd", "inner", "outer", "p2io", "adj_ptr", "adj"):
        assert np.array_equal(ma[k], g["mesh_" + k]), k
    for k in ("xyz", "uv"):
        assert np.array_equal(bits(ma[k]), bits(g["mesh_" + k])), k
    assert o.V == 10 * 4 ** level + 2 and o.T == 20 * 4 ** level
    assert o.os == 1 and o.rs == o.V - 1


def test_operators_bitexact(lvl):
    level, o, g = lvl
    for op in OPS:
        p, c, v = o.csr(op)
        assert np.array_equal(p, g[op + "_ptr"]) and np.array_equal(c, g[op + "_col"]), op
        assert np.array_equal(bits(v), bits(g[op + "_val"])), op


def test_operator_applies(lvl):
    level, o, g = lvl
    u, v, bnd = g["in_u"], g["in_v"], g["in_bnd"]
    assert np.array_equal(bits(o.laplace_calc2(u)), bits(g["out_lap_calc2"]))
    assert np.array_equal(bits(o.laplace_calc1(u, bnd)), bits(g["out_lap_calc1"]))
    assert np.array_equal(bits(o.laplace_solve(u, bnd)), bits(g["out_lap_solve"]))
    assert np.array_equal(bits(o.jacobian_calc2(u, v)), bits(g["out_jac_calc2"]))
    assert np.array_equal(bits(o.jacobian_calc1(u, v, bnd)), bits(g["out_jac_calc1"]))
    n = g["out_norms"]
    assert o.norm(u) == n[0] and o.dist(u, v) == n[1] and o.scalar(u, v) == n[2]


def test_barvortex_steps(lvl):
    level, o, g = lvl
    u = g["in_u"]
    bv = o.barvortex(max_iter=3, coriolis=np.sin(o.mesh_arrays()["uv"].reshape(-1, 4, 2)[:, 0, 0]))
    z = np.zeros(o.os)
    s1 = o.bv_step(bv, u, z, z)
    assert np.array_equal(bits(s1), bits(g["out_bv_step1"]))
    s2 = o.bv_step(bv, s1, z, z)
    assert np.array_equal(bits(s2), bits(g["out_bv_final"]))


def test_baroclin_step(lvl):
    level, o, g = lvl
    lat = o.mesh_arrays()["uv"].reshape(-1, 4, 2)[:, 0, 0]
    bc = o.baroclin(max_iter=3, coriolis=np.sin(lat))
    z = np.zeros(o.os)
    a, b = o.bc_step(bc, g["in_u"], g["in_v"], z)
    assert np.array_equal(bits(a), bits(g["out_bc_step1_u1"]))
    assert np.array_equal(bits(b), bits(g["out_bc_step1_u2"]))


@pytest.mark.parametrize("level", [4, 5])
def test_larger_levels(level, golden):
    """Levels 4-5: mesh topology exact, operator values by digest, applies exact."""
    import hashlib
    g = golden(f"ref_L{level}.npz")
    o = po.Oracle(level)
    ma = o.mesh_arrays()
    for k in ("tri", "tz", "inner", "p2io"):
        assert np.array_equal(ma[k], g["mesh_" + k]), k
    for op in OPS:
        p, c, v = o.csr(op)
        h = hashlib.sha256()
        for a in (p, c, v):
            h.update(np.ascontiguousarray(a).tobytes())
        assert h.hexdigest() == str(g["digest_" + op]), op
    u, v, bnd = g["in_u"], g["in_v"], g["in_bnd"]
    assert np.array_equal(bits(o.laplace_calc1(u, bnd)), bits(g["out_lap_calc1"]))
    assert np.array_equal(bits(o.jacobian_calc2(u, v)), bits(g["out_jac_calc2"]))


# ----------------------------------------------------------- known answers --
def integ(kind, xs, ys, xd, yd, k):
    xs = np.array(xs, float); ys = np.array(ys, float); k = np.array(k, float)
    return po.lib().orc_integrate_poly(kind, po._p(xs), po._p(ys), xd, yd, po._p(k))


def test_kat_integrate():
    # (x - 1)(y - 2) = 2 - x*2... coefficients k[i*(yd+1)+j]: k00=2, k01=-1, k10=-2, k11=1
    k = [2.0, -1.0, -2.0, 1.0]
    tri = ([0.0, 1.0, 1.0], [0.0, 0.0, 1.0])
    assert abs(integ(0, *tri, 1, 1, k) - 0.2916666666666666) <= 1e-14
    assert abs(integ(1, *tri, 1, 1, k) - ((4 * math.sin(1.0) - 9 * math.cos(1.0)) / 2 + 1)) <= 1e-14
    assert abs(integ(2, *tri, 1, 1, k) - (5.0 - (9 * math.sin(1.0) + 4 * math.cos(1.0)) / 2)) <= 1e-14
    assert abs(po.lib().orc_trapezoid_integral(0, 0, 1, 0, 0, 1, 0.5, 1) - 0.125) <= 1e-14


@pytest.mark.parametrize("xs,ys,ans", [
    ([0, 0, math.pi / 8], [0, math.pi / 8, 0], 0.0761204674887130),
    ([0, 0, math.pi / 8], [math.pi / 8, math.pi / 4, math.pi / 8], 0.0761204674887130),
    ([0, math.pi / 8, math.pi / 8], [math.pi / 8, 0, math.pi / 8], 0.0741589649823731),
    ([math.pi / 8, math.pi / 4, math.pi / 8], [0, 0, math.pi / 8], 0.0664933188536525),
])
def test_kat_sphere_area(xs, ys, ans):
    assert abs(integ(1, xs, ys, 0, 0, [1.0]) - ans) <= 1e-14


def test_kat_gauss_kronrod():
    f1 = C.CFUNCTYPE(C.c_double, C.c_double, C.c_void_p)(lambda x, d: x * x)
    f2 = C.CFUNCTYPE(C.c_double, C.c_double, C.c_void_p)(lambda x, d: x / math.cos(x))
    L = po.lib()
    assert abs(L.orc_gauss_kronrod15(0.0, 1.0, C.cast(f1, C.c_void_p), None) - 1.0 / 3.0) <= 1e-14
    assert abs(L.orc_gauss_kronrod15(-1.0, 1.0, C.cast(f2, C.c_void_p), None)) <= 1e-14


@pytest.mark.parametrize("level", [1, 2, 3, 4])
def test_barvortex_linear_steps(golden, level):
    """BarVortex::calc_L / calc_L_1 / calc_LT around z = in_u applied to in_v
    (zero boundary, coriolis sin(lat)): the restatement returns the
    reference's bits."""
    g = golden(f"ref_L{level}.npz")
    o = po.Oracle(level)
    lat = o.mesh_arrays()["uv"].reshape(-1, 4, 2)[:, 0, 0]
    bv = o.barvortex(max_iter=3, coriolis=np.sin(lat))
    z = np.zeros(o.os)
    for which, key in (("L", "out_bv_L"), ("L1", "out_bv_L1"), ("LT", "out_bv_LT")):
        got = o.bv_linear(bv, which, g["in_v"], g["in_u"], z, z)
        assert np.array_equal(bits(got), bits(g[key])), which


@pytest.mark.parametrize("level", [1, 2, 3])
def test_baroclin_linear_steps(golden, level):
    """Baroclin::calc_L / calc_L_1 around (z1, z2) = (in_u, in_v) applied to
    (in_v, in_u), zero boundary: the restatement returns the reference's bits."""
    g = golden(f"ref_L{level}.npz")
    o = po.Oracle(level)
    lat = o.mesh_arrays()["uv"].reshape(-1, 4, 2)[:, 0, 0]
    bc = o.baroclin(max_iter=3, coriolis=np.sin(lat))
    z = np.zeros(o.os)
    for which in ("L", "L1"):
        a, b = o.bc_linear(bc, which, g["in_v"], g["in_u"], g["in_u"], g["in_v"], z)
        assert np.array_equal(bits(a), bits(g[f"out_bc_{which}_u1"])), which
        assert np.array_equal(bits(b), bits(g[f"out_bc_{which}_u2"])), which


@pytest.mark.parametrize("level", [1, 2, 3, 4, 5])
def test_jacobian_adjoint_and_derivatives(golden, level):
    """SphereJacobian::calc1t, calc2_diff_x and calc2_diff_cos_y
    (src/sjacobian.cpp:364-402, 463-468): the restatement returns the
    reference's bits."""
    g = golden(f"ref_L{level}.npz")
    o = po.Oracle(level)
    u, v, bnd = g["in_u"], g["in_v"], g["in_bnd"]
    assert np.array_equal(bits(o.jacobian_calc1t(u, v, bnd)), bits(g["out_jac_calc1t"]))
    assert np.array_equal(bits(o.jacobian_diff_x(u)), bits(g["out_jac_diff_x"]))
    assert np.array_equal(bits(o.jacobian_diff_cos_y(u)), bits(g["out_jac_diff_cos_y"]))


@pytest.mark.parametrize("level", [1, 2, 3, 4])
def test_barvortex_boundary_and_forcing(golden, level):
    """Two BarVortex::calc steps with non-zero pole values (bnd_u, bnd_w) and a
    time-dependent forcing evaluated by the reference at t = 0 and t = tau
    (examples/barvortex_impl.h:171-310): the restatement returns the
    reference's bits."""
    g = golden(f"ref_L{level}.npz")
    o = po.Oracle(level)
    lat = o.mesh_arrays()["uv"].reshape(-1, 4, 2)[:, 0, 0]
    bv = o.barvortex(max_iter=3, coriolis=np.sin(lat))
    bu, bw = g["out_bv_bf_bnd_u"], g["out_bv_bf_bnd_w"]
    assert np.all(bu != 0) and np.all(bw != 0)
    s1 = o.bv_step(bv, g["in_u"], bu, bw, g["out_bv_bf_forcing0"])
    assert np.array_equal(bits(s1), bits(g["out_bv_bf_step1"]))
    s2 = o.bv_step(bv, s1, bu, bw, g["out_bv_bf_forcing1"])
    assert np.array_equal(bits(s2), bits(g["out_bv_bf_step2"]))
