"""The FP32 element-loop quadrature of the Jacobian right-hand sides
(k_jac_quad, phg_jacobian_derivs quad = 1) against the assembled FP64
products (quad = 0) and against host CSR products of the reference's
matrices, levels 3-6, single fields and member batches.

Tolerance: 1e-6 relative L2 per right-hand side for the FP32 quadrature (FP32
gradient weights and 7-point cos rule; the field differences are taken in
FP64 before rounding); the assembled FP64 products agree with the host CSR
products to 1e-14.  The time steps that use the quadrature are checked
end to end in the trajectory, ensemble and baroclinic tests.
"""
import numpy as np
import pytest

from mke_gb300 import fields, phelm

pytestmark = pytest.mark.gpu

# RHS k: (operator, boundary operator, field) in the kernels' order
ORDER = [("d2c", "d2cb", 0), ("d1", "d1b", 1), ("d1c", "d1cb", 0), ("d2", "d2b", 1),
         ("d2", "d2b", 0), ("d1c", "d1cb", 1), ("d1", "d1b", 0), ("d2c", "d2cb", 1)]


def csr_mult(ptr, col, val, x):
    y = np.zeros(len(ptr) - 1)
    for i in range(len(ptr) - 1):
        y[i] = np.dot(val[ptr[i]:ptr[i + 1]], x[col[ptr[i]:ptr[i + 1]]])
    return y


@pytest.mark.parametrize("level", [3, 4, 5, 6])
def test_quadrature_matches_assembled(level):
    import torch
    m = phelm.Mesh.sphere(level)
    lat, lon = m.latlon()
    ops = phelm.Operators(m, phelm.PHG_MIXED)
    J = phelm.SphereJacobian(ops)
    nv = 3
    rng = np.random.default_rng(level)
    U = np.stack([fields.sh_field(fields.random_coeffs(rng, 1, 12), lat, lon) for _ in range(nv)])
    W = np.stack([fields.sh_field(fields.random_coeffs(rng, 1, 12), lat, lon) for _ in range(nv)])
    du, dw = torch.tensor(U, device="cuda"), torch.tensor(W, device="cuda")
    rs = m.inner_size
    a = torch.zeros((nv, 8, rs), dtype=torch.float64, device="cuda")
    q = torch.zeros_like(a)
    J.derivs(du, dw, a, quad=False)
    J.derivs(du, dw, q, quad=True)
    torch.cuda.synchronize()
    a, q = a.cpu().numpy(), q.cpu().numpy()
    for k in range(8):
        for v in range(nv):
            err = np.linalg.norm(q[v, k] - a[v, k]) / np.linalg.norm(a[v, k])
            assert err <= 1e-6, (k, v, err)
    # the assembled products are the reference's matrices applied on the host
    if level <= 5:
        ar = m.arrays()
        isb = ar["bnd"] == 1
        inner_pts = np.flatnonzero(~isb)
        outer_pts = np.flatnonzero(isb)
        for k, (op, bop, f) in enumerate(ORDER):
            x = (U if f == 0 else W)[1]
            y = csr_mult(*m.csr(op), x[inner_pts]) + csr_mult(*m.csr(bop), x[outer_pts])
            assert np.linalg.norm(a[1, k] - y) <= 1e-14 * np.linalg.norm(y), k


def test_quadrature_many_members():
    """256 members (16 member chunks over grid.y) equal the members one by one."""
    import torch
    m = phelm.Mesh.sphere(4)
    lat, lon = m.latlon()
    ops = phelm.Operators(m, phelm.PHG_MIXED)
    J = phelm.SphereJacobian(ops)
    nv = 256
    rng = np.random.default_rng(7)
    base = fields.sh_field(fields.random_coeffs(rng, 1, 10), lat, lon)
    U = np.stack([base * (1 + 0.01 * k) for k in range(nv)])
    W = np.stack([np.roll(base, k) for k in range(nv)])
    du, dw = torch.tensor(U, device="cuda"), torch.tensor(W, device="cuda")
    out = torch.zeros((nv, 8, m.inner_size), dtype=torch.float64, device="cuda")
    J.derivs(du, dw, out, quad=True)
    one = torch.zeros((1, 8, m.inner_size), dtype=torch.float64, device="cuda")
    for k in (0, 15, 16, 255):
        J.derivs(du[k:k + 1], dw[k:k + 1], one, quad=True)
        torch.cuda.synchronize()
        assert torch.equal(out[k], one[0]), k
