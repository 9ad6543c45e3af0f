"""GPU path vs the CPU oracle on the same seeded inputs (through the C ABI).

Tolerances (relative L2 unless stated):
  * operator applies whose only solve is a mass matrix (Laplace calc1/calc2,
    Jacobian calc1/calc2): 1e-13 -- the matrices are bit-identical to the
    reference's and FP64 row sums round like the CPU, so only the mass
    solve's tolerance separates the two;
  * norms / dist / scalar: 1e-13;
  * Laplace solve and barvortex steps: 1e-9, set by the solve tolerance
    (GMRES to 1e-12 relative residual here, the oracle to 1e-13).
"""
import numpy as np
import pytest

import pyoracle as po
from mke_gb300 import fields, phelm

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


_cache = {}


def setup(level, precision=phelm.PHG_FP64):
    key = (level, precision)
    if key not in _cache:
        m = phelm.Mesh.sphere(level)
        ops = phelm.Operators(m, precision, tol=1e-12)
        o = po.Oracle(level)
        lat, lon = m.latlon()
        rng = np.random.default_rng(100 + level)
        u = fields.sh_field(fields.random_coeffs(rng, 1, 8), lat, lon)
        v = fields.sh_field(fields.random_coeffs(rng, 1, 8), lat, lon)
        bnd = u[m.arrays()["bnd"] == 1].copy()
        _cache[key] = (m, ops, o, u, v, bnd, lat, lon)
    return _cache[key]


@pytest.mark.parametrize("level", [2, 3, 4, 5])
def test_laplace_apply(level):
    m, ops, o, u, v, bnd, *_ = setup(level)
    L = phelm.SphereLaplace(ops)
    assert rel(L.calc2(u), o.laplace_calc2(u)) <= 1e-13
    assert rel(L.calc1(u, bnd), o.laplace_calc1(u, bnd)) <= 1e-13


@pytest.mark.parametrize("level", [2, 3, 4, 5])
def test_laplace_solve(level):
    m, ops, o, u, v, bnd, *_ = setup(level)
    L = phelm.SphereLaplace(ops)
    got = L.solve(u, bnd)
    st = ops.last_solve()
    assert st["relres"] <= 1e-12
    assert rel(got, o.laplace_solve(u, bnd)) <= 1e-9
    # round trip through the apply
    assert rel(L.calc1(got, bnd), o.laplace_calc1(o.laplace_solve(u, bnd), bnd)) <= 1e-8


@pytest.mark.parametrize("level", [2, 3, 4, 5])
def test_jacobian(level):
    m, ops, o, u, v, bnd, *_ = setup(level)
    J = phelm.SphereJacobian(ops)
    assert rel(J.calc2(u, v), o.jacobian_calc2(u, v)) <= 1e-13
    assert rel(J.calc1(u, v, bnd), o.jacobian_calc1(u, v, bnd)) <= 1e-13
    assert rel(J.calc2t(u, v), -o.jacobian_calc2(u, v)) <= 1e-13


@pytest.mark.parametrize("level", [2, 4])
def test_norms(level):
    m, ops, o, u, v, bnd, *_ = setup(level)
    N = phelm.SphereNorm(ops)
    assert abs(N.norm(u) - o.norm(u)) <= 1e-13 * o.norm(u)
    assert abs(N.dist(u, v) - o.dist(u, v)) <= 1e-13 * o.dist(u, v)
    assert abs(N.scalar(u, v) - o.scalar(u, v)) <= 1e-13 * abs(o.norm(u) * o.norm(v))


@pytest.mark.parametrize("level,steps", [(2, 2), (3, 2), (4, 1)])
def test_barvortex_steps(level, steps):
    m, ops, o, u, v, bnd, lat, lon = setup(level)
    psi, _ = fields.barvortex_initial(lat, lon, seed=7, lmax_noise=8)
    cor = np.sin(lat)
    bv = phelm.BarVortex(ops, picard_iters=3, coriolis=cor)
    obv = o.barvortex(max_iter=3, coriolis=cor)
    z = np.zeros(m.outer_size)
    a, b = psi.copy(), psi.copy()
    for _ in range(steps):
        a = bv.calc(a, z, z)
        b = o.bv_step(obv, b, z, z)
    assert rel(a, b) <= 1e-9
    st = bv.last_stats()
    assert st["worst_relres"] <= 1e-11


def test_barvortex_batch_equals_single():
    m, ops, o, u, v, bnd, lat, lon = setup(3)
    cor = np.sin(lat)
    bv = phelm.BarVortex(ops, picard_iters=3, coriolis=cor)
    members = np.stack([fields.barvortex_initial(lat, lon, seed=s, lmax_noise=8)[0] for s in range(5)])
    z = np.zeros((5, m.outer_size))
    batch = bv.calc_batch(members, z, z)
    for k in range(5):
        single = bv.calc(members[k], z[k], z[k])
        assert rel(batch[k], single) <= 1e-10


def test_mixed_precision_matches_fp64():
    m, ops, o, u, v, bnd, lat, lon = setup(4)
    mixed = phelm.Operators(m, phelm.PHG_MIXED, tol=1e-12)
    L64, L32 = phelm.SphereLaplace(ops), phelm.SphereLaplace(mixed)
    assert rel(L32.calc2(u), L64.calc2(u)) <= 1e-12
    s64, s32 = L64.solve(u, bnd), L32.solve(u, bnd)
    assert mixed.last_solve()["relres"] <= 1e-12
    assert rel(s32, s64) <= 1e-9
    J64, J32 = phelm.SphereJacobian(ops), phelm.SphereJacobian(mixed)
    assert rel(J32.calc2(u, v), J64.calc2(u, v)) <= 1e-12


@pytest.mark.parametrize("level", [3, 5])
@pytest.mark.parametrize("name", ["idt", "lapl", "jidt", "d1", "d2", "d1c", "d2c"])
def test_operator_apply_bit_exact(level, name):
    """phelm::Solver::mult_vector: the CSR product in ascending column order,
    the same bits as the sequential CPU sum (oracle rounding, no FMA)."""
    m, ops, *_ = setup(level)
    ptr, col, val = m.csr(name)
    n = len(ptr) - 1
    rng = np.random.default_rng(level)
    X = rng.standard_normal((3, n))
    got = ops.mult(name, X)
    W = int(np.diff(ptr).max())
    ref = np.zeros_like(X)
    for k in range(W):   # slot k of every row; rows shorter than k add nothing
        has = np.diff(ptr) > k
        idx = ptr[:-1][has] + k
        ref[:, has] = ref[:, has] + val[idx] * X[:, col[idx]]
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))


def test_operator_apply_fp32():
    torch = pytest.importorskip("torch")
    m, ops, *_ = setup(5, phelm.PHG_MIXED)
    rng = np.random.default_rng(3)
    X = rng.standard_normal((8, m.inner_size))
    ref = ops.mult("lapl", X)
    x = torch.tensor(X.T.copy(), dtype=torch.float32, device="cuda")   # interleaved: rs x nv
    y = torch.empty_like(x)
    ops.mult32("lapl", x, y)
    torch.cuda.synchronize()
    assert rel(y.cpu().numpy().T, ref) <= 1e-5


@pytest.mark.parametrize("level", [2, 3, 4, 5])
def test_jacobian_adjoint_and_derivatives(level, golden):
    """SphereJacobian::calc1t, calc2_diff_x, calc2_diff_cos_y vs the oracle,
    and at levels 2-5 vs the reference's own results (tests/golden).  Each is
    a derivative product and one mass solve: 1e-13."""
    m, ops, o, u, v, bnd, *_ = setup(level)
    J = phelm.SphereJacobian(ops)
    assert rel(J.calc1t(u, v, bnd), o.jacobian_calc1t(u, v, bnd)) <= 1e-13
    assert rel(J.calc1t(u, v, bnd)[m.arrays()["bnd"] == 0], -J.calc1(u, v, bnd)[m.arrays()["bnd"] == 0]) <= 1e-15
    assert rel(J.calc2_diff_x(u), o.jacobian_diff_x(u)) <= 1e-13
    assert rel(J.calc2_diff_cos_y(u), o.jacobian_diff_cos_y(u)) <= 1e-13
    g = golden(f"ref_L{level}.npz")
    gu, gv, gb = g["in_u"], g["in_v"], g["in_bnd"]
    assert rel(J.calc1t(gu, gv, gb), g["out_jac_calc1t"]) <= 1e-13
    assert rel(J.calc2_diff_x(gu), g["out_jac_diff_x"]) <= 1e-13
    assert rel(J.calc2_diff_cos_y(gu), g["out_jac_diff_cos_y"]) <= 1e-13


@pytest.mark.parametrize("precision", [phelm.PHG_FP64, phelm.PHG_MIXED])
@pytest.mark.parametrize("level", [2, 3, 4])
def test_barvortex_boundary_and_forcing(level, precision, golden):
    """Two BarVortex::calc steps with non-zero pole values bnd_u, bnd_w and a
    time-dependent forcing (the reference's own run, tests/golden: forcing
    values as the reference evaluated them at t = 0 and t = tau), single call
    and as a member of a batch.  FP64: 1e-9 (solves to 1e-12).  Mixed: 1e-8 --
    its first two Picard iterations take the Jacobian from the FP32
    quadrature, and on these strongly nonlinear fields (l <= 6, unit
    amplitude, coarse meshes) the third iteration leaves up to 6e-9 of that
    (the FP64 path of the same step: 2e-12)."""
    tol = 1e-9 if precision == phelm.PHG_FP64 else 1e-8
    m, ops, *_ = setup(level, precision)
    g = golden(f"ref_L{level}.npz")
    lat, _ = m.latlon()
    bv = phelm.BarVortex(ops, picard_iters=3, coriolis=np.sin(lat))
    bu, bw = g["out_bv_bf_bnd_u"], g["out_bv_bf_bnd_w"]
    s1 = bv.calc(g["in_u"], bu, bw, forcing=g["out_bv_bf_forcing0"])
    assert rel(s1, g["out_bv_bf_step1"]) <= tol
    s2 = bv.calc(s1, bu, bw, forcing=g["out_bv_bf_forcing1"])
    assert rel(s2, g["out_bv_bf_step2"]) <= tol
    assert bv.last_stats()["worst_relres"] <= 1e-11
    # the same member inside a batch of three (the others: zero boundary)
    U = np.stack([g["in_u"], g["in_v"], g["in_u"]])
    BU = np.stack([np.zeros_like(bu), np.zeros_like(bu), bu])
    BW = np.stack([np.zeros_like(bw), np.zeros_like(bw), bw])
    out = bv.calc_batch(U, BU, BW, forcing=g["out_bv_bf_forcing0"])
    assert rel(out[2], g["out_bv_bf_step1"]) <= tol
