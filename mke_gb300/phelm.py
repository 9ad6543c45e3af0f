"""Python binding of libphelm_gb300 (include/phelm_gb300.h), shaped like the
reference's C++ API: ``Mesh``, ``SphereLaplace``, ``SphereJacobian``,
``SphereNorm``, ``BarVortex``, ``Baroclin``.

Vector arguments are numpy float64 arrays (host memory: the call stages them
to the GPU and returns when the result is back) or CUDA tensors / any object
with ``data_ptr()`` (device memory: the call only enqueues work).  There is no
CPU fallback: without the library or without a GPU the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

PHG_FP64, PHG_MIXED = 0, 1
_ERRORS = {1: "bad argument", 2: "CUDA error", 3: "solve did not converge", 4: "device wait timed out",
           5: "mesh I/O error", 6: "over the HBM budget", 7: "host failure"}
PHG_REQ_LAPLACE_SOLVE, PHG_REQ_BARVORTEX = 0, 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p


class PhgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{_ERRORS.get(code, code)}: {msg}")
        self.code = code


class BvConf(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("tau", "sigma", "mu", "k1", "k2", "theta")] + [("picard_iters", C.c_int)]


class BcConf(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("tau", "sigma", "mu", "sigma1", "mu1", "alpha")] + [
        ("picard_iters", C.c_int), ("picard_tol", C.c_double)]


class ServeConf(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_double), ("precision", C.c_int), ("max_slots", C.c_int),
                ("solve_tol", C.c_double), ("step_tol", C.c_double), ("bv", BvConf)]


class Request(C.Structure):
    _fields_ = [("kind", C.c_int), ("level", C.c_int), ("steps", C.c_int), ("input", _vp), ("bnd", _vp),
                ("output", _vp), ("tag", C.c_longlong)]


class Completion(C.Structure):
    _fields_ = [("tag", C.c_longlong), ("status", C.c_int), ("kind", C.c_int), ("level", C.c_int),
                ("t_submit", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double), ("batch", C.c_int),
                ("error", C.c_char * 128)]


# every symbol the header declares, with its ctypes signature
SIGNATURES = {
    "phg_last_error": (C.c_char_p, []),
    "phg_version": (C.c_char_p, []),
    "phg_kernel_launches": (C.c_longlong, []),
    "phg_mesh_generate": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "phg_mesh_load_file": (C.c_int, [C.c_char_p, C.POINTER(_vp)]),
    "phg_mesh_destroy": (None, [_vp]),
    "phg_cache_dir": (C.c_int, [C.c_char_p]),
    "phg_mesh_save_file": (C.c_int, [_vp, C.c_char_p]),
    "phg_print_function": (C.c_int, [_vp, C.c_char_p, _vp, _vp, _vp, _vp]),
    "phg_print_inner_function": (C.c_int, [_vp, C.c_char_p, _vp, _vp, _vp, _vp]),
    "phg_state_save": (C.c_int, [_vp, C.c_char_p, C.POINTER(_vp), C.c_int, C.c_double, C.c_longlong]),
    "phg_state_load": (C.c_int, [_vp, C.c_char_p, C.POINTER(_vp), C.c_int, _dp, C.POINTER(C.c_longlong)]),
    "phg_mesh_info": (C.c_int, [_vp, _ip, _ip, _ip, _ip]),
    "phg_mesh_arrays": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "phg_mesh_maps": (C.c_int, [_vp, _vp, _vp, _vp]),
    "phg_mesh_csr": (C.c_int, [_vp, C.c_char_p, _ip, _ip, _vp, _vp, _vp]),
    "phg_ops_create": (C.c_int, [_vp, C.c_int, C.POINTER(_vp)]),
    "phg_ops_destroy": (None, [_vp]),
    "phg_ops_set_solver": (C.c_int, [_vp, C.c_int, C.c_double, C.c_int]),
    "phg_ops_last_solve": (C.c_int, [_vp, _ip, _ip, _dp]),
    "phg_ops_profile": (C.c_int, [_vp, C.c_int]),
    "phg_ops_profile_read": (C.c_int, [_vp, _ip, _dp, _dp]),
    "phg_ops_profile_read_family": (C.c_int, [_vp, C.c_int, _ip, _dp, _dp]),
    "phg_laplace_calc1": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "phg_laplace_calc2": (C.c_int, [_vp, _vp, _vp, _vp]),
    "phg_laplace_solve": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "phg_laplace_solve_batch": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _vp]),
    "phg_laplace_solve_levels": (C.c_int, [C.c_int, _vp, _vp, _vp, _vp, _vp, _vp]),
    "phg_ops_check": (C.c_int, [_vp, _vp]),
    "phg_ops_set_sms": (C.c_int, [_vp, C.c_int]),
    "phg_ops_set_wait_limit": (C.c_int, [_vp, C.c_longlong]),
    "phg_ops_mult": (C.c_int, [_vp, C.c_char_p, _vp, _vp, C.c_int, _vp]),
    "phg_ops_mult32": (C.c_int, [_vp, C.c_char_p, _vp, _vp, C.c_int, _vp]),
    "phg_device_bytes": (C.c_int, [C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "phg_laplace_calc2_noalloc": (C.c_int, [_vp, _vp, _vp, _vp]),
    "phg_jacobian_calc1": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "phg_jacobian_calc2": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "phg_jacobian_calc2t": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "phg_jacobian_calc1t": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "phg_jacobian_derivs": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, C.c_int, _vp]),
    "phg_jacobian_calc2_diff_x": (C.c_int, [_vp, _vp, _vp, _vp]),
    "phg_jacobian_calc2_diff_cos_y": (C.c_int, [_vp, _vp, _vp, _vp]),
    "phg_norm": (C.c_int, [_vp, _vp, _dp, _vp]),
    "phg_dist": (C.c_int, [_vp, _vp, _vp, _dp, _vp]),
    "phg_scalar": (C.c_int, [_vp, _vp, _vp, _dp, _vp]),
    "phg_barvortex_create": (C.c_int, [_vp, C.POINTER(BvConf), _vp, C.POINTER(_vp)]),
    "phg_barvortex_destroy": (None, [_vp]),
    "phg_barvortex_calc": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "phg_barvortex_calc_batch": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp]),
    "phg_barvortex_run": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp]),
    "phg_ops_autotune": (C.c_int, [_vp, C.c_int, C.c_char_p, C.c_int, _vp]),
    "phg_ops_validate": (C.c_int, [_vp, C.POINTER(C.c_longlong), _vp]),
    "phg_tune_describe": (C.c_int, [C.c_char_p, C.c_int]),
    "phg_tune_save": (C.c_int, [C.c_char_p]),
    "phg_tune_load": (C.c_int, [C.c_char_p, _ip]),
    "phg_tune_clear": (None, []),
    "phg_barvortex_last_stats": (C.c_int, [_vp, _ip, _ip, _ip, _ip, _dp]),
    "phg_barvortex_calc_L": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "phg_barvortex_calc_L_1": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "phg_barvortex_calc_LT": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "phg_baroclin_create": (C.c_int, [_vp, C.POINTER(BcConf), _vp, C.POINTER(_vp)]),
    "phg_baroclin_destroy": (None, [_vp]),
    "phg_baroclin_calc": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "phg_baroclin_calc_L": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "phg_baroclin_calc_L_1": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "phg_serve_create": (C.c_int, [C.POINTER(ServeConf), C.POINTER(_vp)]),
    "phg_serve_preload": (C.c_int, [_vp, C.c_int, C.c_int]),
    "phg_serve_submit": (C.c_int, [_vp, C.POINTER(Request)]),
    "phg_serve_poll": (C.c_int, [_vp, C.POINTER(Completion), C.c_int, C.c_double, _ip]),
    "phg_serve_stats": (C.c_int, [_vp, _dp, _ip, C.POINTER(C.c_longlong)]),
    "phg_serve_clock": (C.c_double, [_vp]),
    "phg_serve_destroy": (None, [_vp]),
}

_lib = None


def lib(build_if_missing: bool = True):
    """Load (building first if needed) the in-tree library."""
    global _lib
    if _lib is None:
        path = _build.LIB
        if build_if_missing:
            path = _build.build()
        if not os.path.exists(path):
            raise PhgError(2, f"{path} missing (run mke_gb300.build.build())")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def cache_dir(path=None) -> None:
    """Directory of the on-disk level cache (phg_cache_dir); None disables it."""
    _check(lib().phg_cache_dir(path.encode() if path else None))


def tune_table() -> list:
    """The autotuner's table: dicts with kind "solve" (family, rows,
    precision, bucket, rows_per_block, path) or "spmm" (rows, bucket,
    threads_per_row)."""
    buf = C.create_string_buffer(1 << 16)
    _check(lib().phg_tune_describe(buf, len(buf)))
    out = []
    for line in buf.value.decode().splitlines():
        f = line.split()
        if f[0] == "solve":
            out.append(dict(kind="solve", family=int(f[1]), rows=int(f[2]), precision=int(f[3]), bucket=int(f[4]),
                            rows_per_block=int(f[5]), path=int(f[6])))
        elif f[0] == "spmm":
            out.append(dict(kind="spmm", rows=int(f[1]), bucket=int(f[2]), threads_per_row=int(f[3])))
    return out


def tune_save(path: str) -> None:
    _check(lib().phg_tune_save(path.encode()))


def tune_load(path: str) -> int:
    k = C.c_int()
    _check(lib().phg_tune_load(path.encode(), C.byref(k)))
    return k.value


def tune_clear() -> None:
    lib().phg_tune_clear()


def kernel_launches() -> int:
    return int(lib().phg_kernel_launches())


def _check(code):
    if code != 0:
        raise PhgError(code, lib().phg_last_error().decode())


def _ptr(x):
    """Host numpy (float64/int32, C-contiguous) or device tensor -> void*."""
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        return C.c_void_p(x.data_ptr())
    if not isinstance(x, np.ndarray) or not x.flags["C_CONTIGUOUS"]:
        raise TypeError("expected a C-contiguous numpy array or a CUDA tensor")
    return C.c_void_p(x.ctypes.data)


def _f8(x):
    if x is None or hasattr(x, "data_ptr"):
        return x
    return np.ascontiguousarray(x, dtype=np.float64)


def _stream(s):
    if s is None:
        return None
    return C.c_void_p(s if isinstance(s, int) else s.cuda_stream)


class Mesh:
    """phelm::Mesh: ``Mesh.sphere(level)`` or ``Mesh.load(path)``."""

    def __init__(self, handle):
        self._h = handle
        V, T, rs, os_ = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _check(lib().phg_mesh_info(self._h, C.byref(V), C.byref(T), C.byref(rs), C.byref(os_)))
        self.size, self.ntri, self.inner_size, self.outer_size = V.value, T.value, rs.value, os_.value

    @classmethod
    def sphere(cls, level: int) -> "Mesh":
        h = C.c_void_p()
        _check(lib().phg_mesh_generate(level, C.byref(h)))
        return cls(h)

    @classmethod
    def load(cls, path: str) -> "Mesh":
        h = C.c_void_p()
        _check(lib().phg_mesh_load_file(path.encode(), C.byref(h)))
        return cls(h)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.phg_mesh_destroy(self._h)
            self._h = None

    def arrays(self):
        V, T = self.size, self.ntri
        xyz, uv = np.zeros(V * 3), np.zeros(V * 8)
        tri, tz, bnd = np.zeros(T * 3, np.int32), np.zeros(T, np.int32), np.zeros(V, np.int32)
        _check(lib().phg_mesh_arrays(self._h, _ptr(xyz), _ptr(uv), _ptr(tri), _ptr(tz), _ptr(bnd)))
        return {"xyz": xyz, "uv": uv, "tri": tri, "tz": tz, "bnd": bnd}

    def maps(self):
        inner, outer = np.zeros(self.inner_size, np.int32), np.zeros(max(self.outer_size, 1), np.int32)
        p2io = np.zeros(self.size, np.int32)
        _check(lib().phg_mesh_maps(self._h, _ptr(inner), _ptr(outer), _ptr(p2io)))
        return {"inner": inner, "outer": outer[: self.outer_size], "p2io": p2io}

    def save(self, path: str):
        """The reference's mesh text file (as mke_mesh_sphere writes it)."""
        _check(lib().phg_mesh_save_file(self._h, os.fsencode(path)))

    def print_function(self, path: str, ans, x=None, y=None, z=None, inner: bool = False):
        """print_function / print_inner_function of a full vector (host arrays)."""
        ans, x, y, z = _f8(ans), _f8(x), _f8(y), _f8(z)
        fn = lib().phg_print_inner_function if inner else lib().phg_print_function
        _check(fn(self._h, os.fsencode(path), _ptr(ans), _ptr(x), _ptr(y), _ptr(z)))

    def save_state(self, path: str, fields, t: float = 0.0, step: int = 0):
        """Binary checkpoint of full vectors (host arrays) with the model time and step."""
        arrs = [np.ascontiguousarray(f, dtype=np.float64) for f in fields]
        ptrs = (C.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
        _check(lib().phg_state_save(self._h, os.fsencode(path), ptrs, len(arrs), t, step))

    def load_state(self, path: str, nfields: int):
        """(fields, t, step) from a checkpoint written for this mesh."""
        arrs = [np.zeros(self.size) for _ in range(nfields)]
        ptrs = (C.c_void_p * nfields)(*[a.ctypes.data for a in arrs])
        t, st = C.c_double(), C.c_longlong()
        _check(lib().phg_state_load(self._h, os.fsencode(path), ptrs, nfields, C.byref(t), C.byref(st)))
        return arrs, t.value, st.value

    def latlon(self):
        """Zone-0 chart coordinates (latitude, longitude) of every point."""
        uv = self.arrays()["uv"].reshape(-1, 4, 2)
        return uv[:, 0, 0].copy(), uv[:, 0, 1].copy()

    def csr(self, name: str):
        n, nnz = C.c_int(), C.c_int()
        _check(lib().phg_mesh_csr(self._h, name.encode(), C.byref(n), C.byref(nnz), None, None, None))
        ptr, col, val = np.zeros(n.value + 1, np.int32), np.zeros(nnz.value, np.int32), np.zeros(nnz.value)
        _check(lib().phg_mesh_csr(self._h, name.encode(), None, None, _ptr(ptr), _ptr(col), _ptr(val)))
        return ptr, col, val


class Operators:
    """Device-resident SphereLaplace + SphereJacobian + SphereNorm of one mesh."""

    def __init__(self, mesh: Mesh, precision: int = PHG_FP64, restart: int = 30, tol: float = 1e-12,
                 max_iter: int = 20000):
        self.mesh = mesh
        self.precision = precision
        h = C.c_void_p()
        _check(lib().phg_ops_create(mesh._h, precision, C.byref(h)))
        self._h = h
        self.set_solver(restart, tol, max_iter)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.phg_ops_destroy(self._h)
            self._h = None

    def mult(self, name: str, x, out=None, stream=None):
        """phelm::Solver::mult_vector: y = A x on inner vectors (rs or nv x rs)."""
        x = _f8(x)
        nv = 1 if x.ndim == 1 else x.shape[0]
        out = np.zeros_like(x) if out is None else out
        _check(lib().phg_ops_mult(self._h, name.encode(), _ptr(out), _ptr(x), nv, _stream(stream)))
        return out

    def mult32(self, name: str, x, out, stream=None):
        """FP32 operator apply of the mixed path on interleaved multi-vectors
        (CUDA float32 tensors rs x nv, nv = 4 * 2^k <= 256)."""
        _check(lib().phg_ops_mult32(self._h, name.encode(), _ptr(out), _ptr(x), x.shape[1], _stream(stream)))
        return out

    def validate(self, stream=None) -> int:
        """Entries of the handle's device index arrays outside their valid range (0 = all fine)."""
        n = C.c_longlong()
        _check(lib().phg_ops_validate(self._h, C.byref(n), _stream(stream)))
        return n.value

    def autotune(self, members: int = 1, stream=None) -> str:
        """Time the candidate launch shapes of a ``members``-state step's
        kernels and keep the fastest (phg_ops_autotune); returns the report."""
        buf = C.create_string_buffer(1 << 16)
        _check(lib().phg_ops_autotune(self._h, int(members), buf, len(buf), _stream(stream)))
        return buf.value.decode()

    def set_solver(self, restart=30, tol=1e-12, max_iter=20000):
        _check(lib().phg_ops_set_solver(self._h, restart, tol, max_iter))

    def set_sms(self, max_sms: int = 0):
        """Cap the SMs this handle's persistent solver launches use (0 = all)."""
        _check(lib().phg_ops_set_sms(self._h, int(max_sms)))

    def set_wait_limit(self, cycles: int = 0):
        """Clock cycles a group-barrier wait of this handle's persistent solver
        kernels may spin before the launch gives up (0 = the default, ~1 s)."""
        _check(lib().phg_ops_set_wait_limit(self._h, int(cycles)))

    def check(self, stream=None):
        """phg_ops_check: synchronise and check the solves enqueued since the last check."""
        _check(lib().phg_ops_check(self._h, _stream(stream)))

    def profile(self, enable=True):
        _check(lib().phg_ops_profile(self._h, 1 if enable else 0))

    def profile_read(self, family: int = -1):
        """Solver launches recorded since profile(True): count, event-timed ms
        and algorithmic bytes; family restricts to one solver family
        (0 GMRES, 1 Chebyshev, 2 multigrid GMRES, 3 baroclinic block system)."""
        n, ms, b = C.c_int(), C.c_double(), C.c_double()
        _check(lib().phg_ops_profile_read_family(self._h, int(family), C.byref(n), C.byref(ms), C.byref(b)))
        return {"launches": n.value, "ms": ms.value, "bytes": b.value}

    @property
    def stream(self):
        return None

    def last_solve(self):
        it, cy, rr = C.c_int(), C.c_int(), C.c_double()
        _check(lib().phg_ops_last_solve(self._h, C.byref(it), C.byref(cy), C.byref(rr)))
        return {"iters": it.value, "cycles": cy.value, "relres": rr.value}


def _out(like_dev, n):
    return np.zeros(n)


class SphereLaplace:
    """SphereLaplace<double> (src/slaplace.h:60-108): calc1, calc2, solve."""

    def __init__(self, ops: Operators):
        self.ops = ops
        self.m = ops.mesh

    def calc1(self, F, bnd=None, out=None, stream=None):
        out = np.zeros(self.m.size) if out is None else out
        F, bnd = _f8(F), _f8(bnd)
        _check(lib().phg_laplace_calc1(self.ops._h, _ptr(out), _ptr(F), _ptr(bnd), _stream(stream)))
        return out

    def calc2(self, F, out=None, stream=None):
        out = np.zeros(self.m.inner_size) if out is None else out
        F = _f8(F)
        _check(lib().phg_laplace_calc2(self.ops._h, _ptr(out), _ptr(F), _stream(stream)))
        return out

    def solve(self, F, bnd=None, out=None, stream=None):
        out = np.zeros(self.m.size) if out is None else out
        F, bnd = _f8(F), _f8(bnd)
        _check(lib().phg_laplace_solve(self.ops._h, _ptr(out), _ptr(F), _ptr(bnd), _stream(stream)))
        return out

    def solve_batch(self, F, bnd=None, out=None, stream=None):
        """nv right-hand sides (nv x V, member-major) in one launch."""
        nv = F.shape[0]
        out = np.zeros((nv, self.m.size)) if out is None else out
        F, bnd = _f8(F), _f8(bnd)
        _check(lib().phg_laplace_solve_batch(self.ops._h, nv, _ptr(out), _ptr(F), _ptr(bnd), _stream(stream)))
        return out


class SphereJacobian:
    """SphereJacobian (src/sjacobian.h:65-149): calc1, calc1t, calc2, calc2t,
    calc2_diff_x, calc2_diff_cos_y."""

    def __init__(self, ops: Operators):
        self.ops = ops
        self.m = ops.mesh

    def calc1(self, u, v, bnd=None, out=None, stream=None):
        out = np.zeros(self.m.size) if out is None else out
        u, v, bnd = _f8(u), _f8(v), _f8(bnd)
        _check(lib().phg_jacobian_calc1(self.ops._h, _ptr(out), _ptr(u), _ptr(v), _ptr(bnd), _stream(stream)))
        return out

    def calc2(self, u, v, out=None, stream=None):
        out = np.zeros(self.m.inner_size) if out is None else out
        u, v = _f8(u), _f8(v)
        _check(lib().phg_jacobian_calc2(self.ops._h, _ptr(out), _ptr(u), _ptr(v), _stream(stream)))
        return out

    def calc2t(self, u, v, out=None, stream=None):
        out = np.zeros(self.m.inner_size) if out is None else out
        u, v = _f8(u), _f8(v)
        _check(lib().phg_jacobian_calc2t(self.ops._h, _ptr(out), _ptr(u), _ptr(v), _stream(stream)))
        return out

    def derivs(self, u, v, out, quad=False, stream=None):
        """The 8 derivative products of calc2 (CUDA float64 tensors: u, v
        nv x V, out nv x 8 x rs); quad: the FP32 element-loop quadrature."""
        nv = 1 if u.dim() == 1 else u.shape[0]
        _check(lib().phg_jacobian_derivs(self.ops._h, 1 if quad else 0, _ptr(out), _ptr(u), _ptr(v), nv,
                                         _stream(stream)))
        return out

    def calc1t(self, u, v, bnd=None, out=None, stream=None):
        """SphereJacobian::calc1t: -J(u, v) on the inner points, bnd on the boundary."""
        out = np.zeros(self.m.size) if out is None else out
        u, v, bnd = _f8(u), _f8(v), _f8(bnd)
        _check(lib().phg_jacobian_calc1t(self.ops._h, _ptr(out), _ptr(u), _ptr(v), _ptr(bnd), _stream(stream)))
        return out

    def calc2_diff_x(self, v, out=None, stream=None):
        """SphereJacobian::calc2_diff_x: dv/dx on the inner points."""
        out = np.zeros(self.m.inner_size) if out is None else out
        v = _f8(v)
        _check(lib().phg_jacobian_calc2_diff_x(self.ops._h, _ptr(out), _ptr(v), _stream(stream)))
        return out

    def calc2_diff_cos_y(self, v, out=None, stream=None):
        """SphereJacobian::calc2_diff_cos_y: (1/cos y) dv/dy on the inner points."""
        out = np.zeros(self.m.inner_size) if out is None else out
        v = _f8(v)
        _check(lib().phg_jacobian_calc2_diff_cos_y(self.ops._h, _ptr(out), _ptr(v), _stream(stream)))
        return out


class SphereNorm:
    """SphereNorm<double> (src/norm.h:58-120): norm, dist, scalar."""

    def __init__(self, ops: Operators):
        self.ops = ops

    def norm(self, u, stream=None):
        r = C.c_double()
        _check(lib().phg_norm(self.ops._h, _ptr(_f8(u)), C.byref(r), _stream(stream)))
        return r.value

    def dist(self, u, v, stream=None):
        r = C.c_double()
        _check(lib().phg_dist(self.ops._h, _ptr(_f8(u)), _ptr(_f8(v)), C.byref(r), _stream(stream)))
        return r.value

    def scalar(self, u, v, stream=None):
        r = C.c_double()
        _check(lib().phg_scalar(self.ops._h, _ptr(_f8(u)), _ptr(_f8(v)), C.byref(r), _stream(stream)))
        return r.value


class BarVortex:
    """SBarVortex (examples/barvortex.h:109-241): calc (one step), plus calc_batch."""

    def __init__(self, ops: Operators, tau=1e-3, sigma=1.6e-2, mu=8e-5, k1=1.0, k2=1.0, theta=0.5,
                 picard_iters=3, coriolis=None):
        self.ops = ops
        self.m = ops.mesh
        c = BvConf(tau, sigma, mu, k1, k2, theta, picard_iters)
        cor = _f8(coriolis)
        h = C.c_void_p()
        _check(lib().phg_barvortex_create(ops._h, C.byref(c), _ptr(cor), C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.phg_barvortex_destroy(self._h)
            self._h = None

    def calc(self, u, bnd_u=None, bnd_w=None, forcing=None, out=None, stream=None):
        out = np.zeros(self.m.size) if out is None else out
        u, bnd_u, bnd_w, forcing = _f8(u), _f8(bnd_u), _f8(bnd_w), _f8(forcing)
        _check(lib().phg_barvortex_calc(self._h, _ptr(out), _ptr(u), _ptr(bnd_u), _ptr(bnd_w), _ptr(forcing),
                                        _stream(stream)))
        return out

    def calc_batch(self, u, bnd_u=None, bnd_w=None, forcing=None, out=None, stream=None):
        """u: members x V (member-major)."""
        nm = u.shape[0]
        out = np.zeros((nm, self.m.size)) if out is None else out
        u, bnd_u, bnd_w, forcing = _f8(u), _f8(bnd_u), _f8(bnd_w), _f8(forcing)
        _check(lib().phg_barvortex_calc_batch(self._h, nm, _ptr(out), _ptr(u), _ptr(bnd_u), _ptr(bnd_w),
                                              _ptr(forcing), _stream(stream)))
        return out

    def run(self, u, steps, bnd_u=None, bnd_w=None, forcing=None, stream=None):
        """``steps`` steps of u in place (V values, or members x V), the same
        boundary values and forcing every step; after the first step each
        step is one launch of a captured CUDA graph.  Host arrays must be
        writable float64 C-contiguous."""
        nm = 1 if u.ndim == 1 else u.shape[0]
        if not hasattr(u, "data_ptr") and (u.dtype != np.float64 or not u.flags.c_contiguous):
            raise TypeError("u must be a C-contiguous float64 array (updated in place)")
        bnd_u, bnd_w, forcing = _f8(bnd_u), _f8(bnd_w), _f8(forcing)
        _check(lib().phg_barvortex_run(self._h, nm, int(steps), _ptr(u), _ptr(bnd_u), _ptr(bnd_w), _ptr(forcing),
                                       _stream(stream)))
        return u

    def _linear(self, fn, u, z, bnd_u, bnd_w, out, stream):
        out = np.zeros(self.m.size) if out is None else out
        u, z = _f8(u), _f8(z)
        _check(getattr(lib(), fn)(self._h, _ptr(out), _ptr(u), _ptr(z), _ptr(_f8(bnd_u)), _ptr(_f8(bnd_w)),
                                  _stream(stream)))
        return out

    def calc_L(self, u, z, bnd_u=None, bnd_w=None, out=None, stream=None):
        """BarVortex::calc_L: the step linearised around z, applied to u."""
        return self._linear("phg_barvortex_calc_L", u, z, bnd_u, bnd_w, out, stream)

    def calc_L_1(self, u, z, bnd_u=None, bnd_w=None, out=None, stream=None):
        """BarVortex::calc_L_1: inverse linearised step; adds into ``out`` (zeros when None)."""
        return self._linear("phg_barvortex_calc_L_1", u, z, bnd_u, bnd_w, out, stream)

    def calc_LT(self, v, z, bnd_u=None, bnd_w=None, out=None, stream=None):
        """BarVortex::calc_LT: adjoint of the linearised step around z, applied to v."""
        return self._linear("phg_barvortex_calc_LT", v, z, bnd_u, bnd_w, out, stream)

    def last_stats(self):
        a = [C.c_int() for _ in range(4)]
        w = C.c_double()
        _check(lib().phg_barvortex_last_stats(self._h, *[C.byref(x) for x in a], C.byref(w)))
        return {"iters_lapl": a[0].value, "iters_a": a[1].value, "iters_mj": a[2].value, "iters_ml": a[3].value,
                "worst_relres": w.value}


class Baroclin:
    """Baroclin (examples/baroclin.h:78-287): calc (one step)."""

    def __init__(self, ops: Operators, tau=1e-3, sigma=0.05, mu=6.77e-5, sigma1=0.05, mu1=6.77e-5,
                 alpha=0.1 ** 0.5, picard_iters=3, picard_tol=1e-8, coriolis=None):
        self.ops = ops
        self.m = ops.mesh
        c = BcConf(tau, sigma, mu, sigma1, mu1, alpha, picard_iters, picard_tol)
        h = C.c_void_p()
        _check(lib().phg_baroclin_create(ops._h, C.byref(c), _ptr(_f8(coriolis)), C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.phg_baroclin_destroy(self._h)
            self._h = None

    def calc(self, u1, u2, bnd=None, f=None, g=None, out1=None, out2=None, stream=None):
        out1 = np.zeros(self.m.size) if out1 is None else out1
        out2 = np.zeros(self.m.size) if out2 is None else out2
        _check(lib().phg_baroclin_calc(self._h, _ptr(out1), _ptr(out2), _ptr(_f8(u1)), _ptr(_f8(u2)),
                                       _ptr(_f8(bnd)), _ptr(_f8(f)), _ptr(_f8(g)), _stream(stream)))
        return out1, out2

    def _linear(self, fn, u1, u2, z1, z2, bnd, out1, out2, stream):
        out1 = np.zeros(self.m.size) if out1 is None else out1
        out2 = np.zeros(self.m.size) if out2 is None else out2
        _check(getattr(lib(), fn)(self._h, _ptr(out1), _ptr(out2), _ptr(_f8(u1)), _ptr(_f8(u2)), _ptr(_f8(z1)),
                                  _ptr(_f8(z2)), _ptr(_f8(bnd)), _stream(stream)))
        return out1, out2

    def calc_L(self, u1, u2, z1, z2, bnd=None, out1=None, out2=None, stream=None):
        """Baroclin::calc_L: the step linearised around (z1, z2)."""
        return self._linear("phg_baroclin_calc_L", u1, u2, z1, z2, bnd, out1, out2, stream)

    def calc_L_1(self, u1, u2, z1, z2, bnd=None, out1=None, out2=None, stream=None):
        """Baroclin::calc_L_1: the inverse linearised step around (z1, z2)."""
        return self._linear("phg_baroclin_calc_L_1", u1, u2, z1, z2, bnd, out1, out2, stream)


def laplace_solve_levels(ops_list, F_list, bnd_list=None, stream=None):
    """SphereLaplace::solve for right-hand sides on meshes of several levels in
    one persistent launch (phg_laplace_solve_levels): ops_list[k] an Operators
    handle, F_list[k] its nv_k x V_k right-hand sides (numpy arrays or CUDA
    tensors); returns the solutions in the same layout."""
    n = len(ops_list)
    outs, Fs, Bs, keep = [], [], [], []
    for k, (o, F) in enumerate(zip(ops_list, F_list)):
        F2 = F if hasattr(F, "data_ptr") else _f8(np.atleast_2d(F))
        keep.append(F2)
        outs.append(np.zeros((F2.shape[0], o.mesh.size)) if not hasattr(F2, "data_ptr") else F2.new_zeros(F2.shape))
        b = None if bnd_list is None else bnd_list[k]
        if b is not None and not hasattr(b, "data_ptr"):
            b = _f8(np.atleast_2d(b))
        keep.append(b)
        Fs.append(_ptr(F2)); Bs.append(_ptr(b))
    h = (C.c_void_p * n)(*[o._h for o in ops_list])
    nv = (C.c_int * n)(*[int(f.shape[0]) for f in keep[0::2]])
    ans = (C.c_void_p * n)(*[_ptr(o) for o in outs])
    fp = (C.c_void_p * n)(*Fs)
    bp = (C.c_void_p * n)(*Bs)
    _check(lib().phg_laplace_solve_levels(n, h, nv, ans, fp, bp if bnd_list is not None else None, _stream(stream)))
    return outs


def device_bytes():
    """(total, this thread) device bytes the library holds."""
    t, m = C.c_longlong(), C.c_longlong()
    _check(lib().phg_device_bytes(C.byref(t), C.byref(m)))
    return t.value, m.value


class Server:
    """Request loop with continuous batching (phg_serve_*).

    ``submit`` takes host numpy arrays; they are kept alive here until the
    request's completion has been polled, and ``poll`` returns dicts with the
    completion fields plus ``output`` (the array the result was written to).
    """

    def __init__(self, precision=PHG_MIXED, hbm_budget_bytes=150e9, max_slots=64, solve_tol=1e-10,
                 step_tol=1e-12, tau=1e-3, sigma=1.6e-2, mu=8e-5, k1=1.0, k2=1.0, theta=0.5, picard_iters=3):
        bv = BvConf(tau, sigma, mu, k1, k2, theta, picard_iters)
        c = ServeConf(hbm_budget_bytes, precision, max_slots, solve_tol, step_tol, bv)
        h = C.c_void_p()
        _check(lib().phg_serve_create(C.byref(c), C.byref(h)))
        self._h = h
        self._live = {}
        self._buf = (Completion * 256)()

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.phg_serve_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def clock(self) -> float:
        return lib().phg_serve_clock(self._h)

    def preload(self, kind: int, level: int):
        _check(lib().phg_serve_preload(self._h, kind, level))

    def submit(self, kind: int, level: int, input, bnd=None, steps: int = 1, tag: int = 0, output=None):
        inp = np.ascontiguousarray(input, dtype=np.float64)
        b = None if bnd is None else np.ascontiguousarray(bnd, dtype=np.float64)
        out = np.empty_like(inp) if output is None else output
        r = Request(kind, level, steps, inp.ctypes.data, None if b is None else b.ctypes.data, out.ctypes.data, tag)
        self._live[tag] = (inp, b, out)
        _check(lib().phg_serve_submit(self._h, C.byref(r)))

    def poll(self, wait: float = 0.0, max_n: int = 256):
        n = C.c_int()
        _check(lib().phg_serve_poll(self._h, self._buf, min(max_n, 256), wait, C.byref(n)))
        res = []
        for k in range(n.value):
            c = self._buf[k]
            keep = self._live.pop(c.tag, None)
            res.append({"tag": c.tag, "status": c.status, "kind": c.kind, "level": c.level,
                        "t_submit": c.t_submit, "t_admit": c.t_admit, "t_done": c.t_done, "batch": c.batch,
                        "error": c.error.decode(errors="replace"),
                        "output": keep[2] if keep else None})
        return res

    def stats(self):
        b, nl, d = C.c_double(), C.c_int(), C.c_longlong()
        _check(lib().phg_serve_stats(self._h, C.byref(b), C.byref(nl), C.byref(d)))
        return {"bytes_in_use": b.value, "lanes": nl.value, "completed": d.value}
