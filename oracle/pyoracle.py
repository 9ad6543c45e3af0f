"""ctypes loader for the CPU oracle (oracle/_build/libphelm_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py`` -- never by the product package.
The oracle restates the reference's sphere-FEM algorithm in C (see
``phelm_oracle.h``); this module only marshals arrays.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libphelm_oracle.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Csr(C.Structure):
    _fields_ = [("n", C.c_int), ("m", C.c_int), ("ptr", _ip), ("col", _ip),
                ("val", _dp), ("ilu", _dp), ("diag", _ip)]

    def arrays(self):
        nnz = self.ptr[self.n]
        ptr = np.ctypeslib.as_array(self.ptr, (self.n + 1,)).copy()
        col = np.ctypeslib.as_array(self.col, (max(nnz, 1),))[:nnz].copy()
        val = np.ctypeslib.as_array(self.val, (max(nnz, 1),))[:nnz].copy()
        return ptr, col, val


class Mesh(C.Structure):
    _fields_ = [("V", C.c_int), ("T", C.c_int), ("xyz", _dp), ("uv", _dp), ("nz", C.c_int),
                ("tri", _ip), ("tz", _ip), ("bnd", _ip), ("rs", C.c_int), ("os", C.c_int),
                ("inner", _ip), ("outer", _ip), ("p2io", _ip), ("adj_ptr", _ip), ("adj", _ip)]


class Ops(C.Structure):
    _fields_ = [("m", C.POINTER(Mesh))] + [(n, Csr) for n in (
        "idt", "lapl", "bnd1", "bnd2", "bnd3", "jidt", "d1", "d2", "d1c", "d2c",
        "d1b", "d2b", "d1cb", "d2cb", "norm")]


class BvConf(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("tau", "sigma", "mu", "k1", "k2", "theta")] + [
        ("max_iter", C.c_int)]


class BarVortex(C.Structure):
    _fields_ = [("o", C.POINTER(Ops)), ("c", BvConf), ("A", Csr), ("bndA", Csr), ("Ab", Csr), ("bndAb", Csr),
                ("lh", _dp), ("last_iters", C.c_int)]


class BcConf(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("tau", "sigma", "mu", "sigma1", "mu1", "alpha", "theta")] + [
        ("max_iter", C.c_int), ("tol", C.c_double)]


class Baroclin(C.Structure):
    _fields_ = [("o", C.POINTER(Ops)), ("c", BcConf), ("A", Csr), ("Ab", Csr), ("lh", _dp),
                ("last_iters", C.c_int)]


def build():
    """Compile the oracle library (plain make; gcc only)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_mesh_sphere.argtypes = [C.POINTER(Mesh), C.c_int]
        L.orc_ops_build.argtypes = [C.POINTER(Ops), C.POINTER(Mesh)]
        for f in ("orc_laplace_calc2",):
            getattr(L, f).argtypes = [C.POINTER(Ops), _dp, _dp]
        L.orc_laplace_calc1.argtypes = [C.POINTER(Ops), _dp, _dp, _dp]
        L.orc_laplace_solve.argtypes = [C.POINTER(Ops), _dp, _dp, _dp]
        L.orc_jacobian_calc2.argtypes = [C.POINTER(Ops), _dp, _dp, _dp]
        L.orc_jacobian_calc1.argtypes = [C.POINTER(Ops), _dp, _dp, _dp, _dp]
        L.orc_jacobian_calc1t.argtypes = [C.POINTER(Ops), _dp, _dp, _dp, _dp]
        L.orc_jacobian_diff_x.argtypes = [C.POINTER(Ops), _dp, _dp]
        L.orc_jacobian_diff_cos_y.argtypes = [C.POINTER(Ops), _dp, _dp]
        for f in ("orc_norm",):
            getattr(L, f).argtypes = [C.POINTER(Ops), _dp]
            getattr(L, f).restype = C.c_double
        for f in ("orc_dist", "orc_scalar"):
            getattr(L, f).argtypes = [C.POINTER(Ops), _dp, _dp]
            getattr(L, f).restype = C.c_double
        L.orc_bv_init.argtypes = [C.POINTER(BarVortex), C.POINTER(Ops), C.POINTER(BvConf), _dp]
        L.orc_bv_step.argtypes = [C.POINTER(BarVortex), _dp, _dp, _dp, _dp, _dp]
        for f in ("orc_bv_calc_L", "orc_bv_calc_L1", "orc_bv_calc_LT"):
            getattr(L, f).argtypes = [C.POINTER(BarVortex), _dp, _dp, _dp, _dp, _dp]
        L.orc_bc_init.argtypes = [C.POINTER(Baroclin), C.POINTER(Ops), C.POINTER(BcConf), _dp]
        L.orc_bc_step.argtypes = [C.POINTER(Baroclin), _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        for f in ("orc_bc_calc_L", "orc_bc_calc_L1"):
            getattr(L, f).argtypes = [C.POINTER(Baroclin), _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_set_solver.argtypes = [C.c_double, C.c_int, C.c_int]
        L.orc_last_residual.restype = C.c_double
        L.orc_gauss_kronrod15.restype = C.c_double
        L.orc_gauss_kronrod15.argtypes = [C.c_double, C.c_double, C.c_void_p, C.c_void_p]
        L.orc_trapezoid_integral.restype = C.c_double
        L.orc_trapezoid_integral.argtypes = [C.c_int, C.c_int] + [C.c_double] * 6
        L.orc_integrate_poly.restype = C.c_double
        L.orc_integrate_poly.argtypes = [C.c_int, _dp, _dp, C.c_int, C.c_int, _dp]
        L.orc_csr_solve.argtypes = [C.POINTER(Csr), _dp, _dp]
        L.orc_csr_mult.argtypes = [C.POINTER(Csr), _dp, _dp]
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    return a.ctypes.data_as(_dp)


def _f8(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Oracle:
    """One level of the oracle: mesh + operators (+ optional models)."""

    def __init__(self, level: int):
        L = lib()
        self.level = level
        self.mesh = Mesh()
        if L.orc_mesh_sphere(C.byref(self.mesh), level) != 0:
            raise ValueError("bad level")
        self.ops = Ops()
        L.orc_ops_build(C.byref(self.ops), C.byref(self.mesh))
        m = self.mesh
        self.V, self.T, self.rs, self.os = m.V, m.T, m.rs, m.os

    # ---- mesh arrays ----
    def mesh_arrays(self):
        m = self.mesh
        g = np.ctypeslib.as_array
        return {
            "xyz": g(m.xyz, (m.V * 3,)).copy(), "uv": g(m.uv, (m.V * 8,)).copy(),
            "tri": g(m.tri, (m.T * 3,)).copy(), "tz": g(m.tz, (m.T,)).copy(),
            "bnd": g(m.bnd, (m.V,)).copy(), "inner": g(m.inner, (max(m.rs, 1),))[:m.rs].copy(),
            "outer": g(m.outer, (max(m.os, 1),))[:m.os].copy(), "p2io": g(m.p2io, (m.V,)).copy(),
            "adj_ptr": g(m.adj_ptr, (m.V + 1,)).copy(), "adj": g(m.adj, (m.T * 3,)).copy(),
        }

    def csr(self, name):
        return getattr(self.ops, name).arrays()

    # ---- operators ----
    def laplace_calc2(self, F):
        out = np.zeros(self.rs)
        lib().orc_laplace_calc2(C.byref(self.ops), _p(out), _p(_f8(F)))
        return out

    def laplace_calc1(self, F, bnd=None):
        out = np.zeros(self.V)
        lib().orc_laplace_calc1(C.byref(self.ops), _p(out), _p(_f8(F)), _p(None if bnd is None else _f8(bnd)))
        return out

    def laplace_solve(self, F, bnd=None):
        out = np.zeros(self.V)
        lib().orc_laplace_solve(C.byref(self.ops), _p(out), _p(_f8(F)), _p(None if bnd is None else _f8(bnd)))
        return out

    def jacobian_calc2(self, u, v):
        out = np.zeros(self.rs)
        lib().orc_jacobian_calc2(C.byref(self.ops), _p(out), _p(_f8(u)), _p(_f8(v)))
        return out

    def jacobian_calc1(self, u, v, bnd=None):
        out = np.zeros(self.V)
        lib().orc_jacobian_calc1(C.byref(self.ops), _p(out), _p(_f8(u)), _p(_f8(v)),
                                 _p(None if bnd is None else _f8(bnd)))
        return out

    def jacobian_calc1t(self, u, v, bnd=None):
        out = np.zeros(self.V)
        lib().orc_jacobian_calc1t(C.byref(self.ops), _p(out), _p(_f8(u)), _p(_f8(v)),
                                  _p(None if bnd is None else _f8(bnd)))
        return out

    def jacobian_diff_x(self, v):
        out = np.zeros(self.rs)
        lib().orc_jacobian_diff_x(C.byref(self.ops), _p(out), _p(_f8(v)))
        return out

    def jacobian_diff_cos_y(self, v):
        out = np.zeros(self.rs)
        lib().orc_jacobian_diff_cos_y(C.byref(self.ops), _p(out), _p(_f8(v)))
        return out

    def norm(self, u):
        return lib().orc_norm(C.byref(self.ops), _p(_f8(u)))

    def dist(self, u, v):
        return lib().orc_dist(C.byref(self.ops), _p(_f8(u)), _p(_f8(v)))

    def scalar(self, u, v):
        return lib().orc_scalar(C.byref(self.ops), _p(_f8(u)), _p(_f8(v)))

    # ---- models ----
    def barvortex(self, tau=1e-3, sigma=1.6e-2, mu=8e-5, k1=1.0, k2=1.0, theta=0.5,
                  max_iter=3, coriolis=None):
        c = BvConf(tau, sigma, mu, k1, k2, theta, max_iter)
        bv = BarVortex()
        cor = None if coriolis is None else _f8(coriolis)
        lib().orc_bv_init(C.byref(bv), C.byref(self.ops), C.byref(c), _p(cor))
        bv._keep = (self, cor)
        return bv

    def bv_step(self, bv, u, bnd_u=None, bnd_w=None, rp=None):
        out = np.zeros(self.V)
        lib().orc_bv_step(C.byref(bv), _p(out), _p(_f8(u)),
                          _p(None if bnd_u is None else _f8(bnd_u)),
                          _p(None if bnd_w is None else _f8(bnd_w)),
                          _p(None if rp is None else _f8(rp)))
        return out

    def bv_linear(self, bv, which, u, z, bnd_u=None, bnd_w=None, u1=None):
        """BarVortex::calc_L ("L"), calc_L_1 ("L1", adds into u1) or calc_LT ("LT")."""
        out = np.zeros(self.V) if u1 is None else np.array(u1, dtype=np.float64)
        fn = {"L": "orc_bv_calc_L", "L1": "orc_bv_calc_L1", "LT": "orc_bv_calc_LT"}[which]
        getattr(lib(), fn)(C.byref(bv), _p(out), _p(_f8(u)), _p(_f8(z)),
                           _p(None if bnd_u is None else _f8(bnd_u)), _p(None if bnd_w is None else _f8(bnd_w)))
        return out

    def baroclin(self, tau=1e-3, sigma=0.05, mu=6.77e-5, sigma1=0.05, mu1=6.77e-5,
                 alpha=0.1 ** 0.5, theta=0.5, max_iter=3, tol=1e-8, coriolis=None):
        c = BcConf(tau, sigma, mu, sigma1, mu1, alpha, theta, max_iter, tol)
        bc = Baroclin()
        cor = None if coriolis is None else _f8(coriolis)
        lib().orc_bc_init(C.byref(bc), C.byref(self.ops), C.byref(c), _p(cor))
        bc._keep = (self, cor)
        return bc

    def bc_linear(self, bc, which, u1, u2, z1, z2, bnd=None):
        """Baroclin::calc_L ("L") or calc_L_1 ("L1") around (z1, z2)."""
        o1, o2 = np.zeros(self.V), np.zeros(self.V)
        fn = {"L": "orc_bc_calc_L", "L1": "orc_bc_calc_L1"}[which]
        getattr(lib(), fn)(C.byref(bc), _p(o1), _p(o2), _p(_f8(u1)), _p(_f8(u2)), _p(_f8(z1)), _p(_f8(z2)),
                           _p(None if bnd is None else _f8(bnd)))
        return o1, o2

    def bc_step(self, bc, u1, u2, bnd=None, f=None, g=None):
        o1, o2 = np.zeros(self.V), np.zeros(self.V)
        lib().orc_bc_step(C.byref(bc), _p(o1), _p(o2), _p(_f8(u1)), _p(_f8(u2)),
                          _p(None if bnd is None else _f8(bnd)),
                          _p(None if f is None else _f8(f)), _p(None if g is None else _f8(g)))
        return o1, o2


def set_solver(rel_tol=1e-13, restart=60, max_iter=40000):
    lib().orc_set_solver(rel_tol, restart, max_iter)
