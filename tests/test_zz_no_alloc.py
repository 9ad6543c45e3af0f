"""The no-allocation Laplace apply (phg_laplace_calc2_noalloc) against the
regular one (phg_laplace_calc2), through the C ABI.

Some callers cannot let a library allocate device memory (their memory is
owned by their own pool or allocator, or a cudaMalloc's device
synchronisation would stall their other streams); this entry point serves
them from a fixed device array inside the library.  Two calls in a row must
each match the regular entry point within the apply tolerance of the parity
tests (1e-13 relative L2); host pointers and workspaces beyond the array's
16 MiB are refused, and a mass solve that fails (a NaN input) is reported by
phg_ops_check like any other.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from mke_gb300 import fields, phelm

pytestmark = pytest.mark.gpu


def test_laplace_calc2_noalloc_matches_calc2():
    import torch
    L = phelm.lib()
    m = phelm.Mesh.sphere(5)
    ops = phelm.Operators(m, phelm.PHG_FP64, tol=1e-12)
    lat, lon = m.latlon()
    F = fields.sh_field(fields.random_coeffs(np.random.default_rng(11), 1, 8), lat, lon)
    want = phelm.SphereLaplace(ops).calc2(F)
    s = torch.cuda.Stream()
    dF = torch.tensor(F, dtype=torch.float64, device="cuda")
    for k in range(2):
        out = torch.full((m.inner_size,), float("nan"), dtype=torch.float64, device="cuda")
        rc = L.phg_laplace_calc2_noalloc(ops._h, C.c_void_p(out.data_ptr()), C.c_void_p(dF.data_ptr()),
                                         C.c_void_p(s.cuda_stream))
        assert rc == 0, L.phg_last_error().decode()
        s.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert np.linalg.norm(got - want) / np.linalg.norm(want) <= 1e-13, k


def test_laplace_calc2_noalloc_refusals():
    L = phelm.lib()
    m = phelm.Mesh.sphere(3)
    ops = phelm.Operators(m, phelm.PHG_FP64)
    F = np.zeros(m.size)
    out = np.zeros(m.inner_size)
    rc = L.phg_laplace_calc2_noalloc(ops._h, C.c_void_p(out.ctypes.data), C.c_void_p(F.ctypes.data), None)
    assert rc == phelm.PhgError(1, "").code and "device pointers" in L.phg_last_error().decode()


def test_laplace_calc2_noalloc_rejects_oversize(monkeypatch):
    """A mass solve by GMRES(48) at level 6 needs more than the 16 MiB scratch
    (with the default Chebyshev solve the same call fits: four vectors)."""
    import torch
    L = phelm.lib()
    m = phelm.Mesh.sphere(6)
    monkeypatch.setenv("PHG_CHEB", "0")        # read when the operators are built
    ops = phelm.Operators(m, phelm.PHG_FP64, restart=48)
    monkeypatch.delenv("PHG_CHEB")
    dF = torch.zeros(m.size, dtype=torch.float64, device="cuda")
    out = torch.zeros(m.inner_size, dtype=torch.float64, device="cuda")
    rc = L.phg_laplace_calc2_noalloc(ops._h, C.c_void_p(out.data_ptr()), C.c_void_p(dF.data_ptr()), None)
    assert rc == 1 and "16 MiB" in L.phg_last_error().decode()


def test_laplace_calc2_noalloc_reports_failed_solve():
    """The call only enqueues work; its mass solve's record goes to the
    handle, so phg_ops_check reports a NaN input as PHG_ERR_NOT_CONVERGED and
    a clean call after it as PHG_OK."""
    import torch
    L = phelm.lib()
    m = phelm.Mesh.sphere(4)
    ops = phelm.Operators(m, phelm.PHG_FP64, tol=1e-12)
    lat, lon = m.latlon()
    F = fields.sh_field(fields.random_coeffs(np.random.default_rng(12), 1, 8), lat, lon)
    s = torch.cuda.Stream()
    out = torch.zeros(m.inner_size, dtype=torch.float64, device="cuda")
    bad = F.copy()
    bad[40] = np.nan
    dbad = torch.tensor(bad, dtype=torch.float64, device="cuda")
    rc = L.phg_laplace_calc2_noalloc(ops._h, C.c_void_p(out.data_ptr()), C.c_void_p(dbad.data_ptr()),
                                     C.c_void_p(s.cuda_stream))
    assert rc == 0, L.phg_last_error().decode()
    assert L.phg_ops_check(ops._h, C.c_void_p(s.cuda_stream)) == 3
    dF = torch.tensor(F, dtype=torch.float64, device="cuda")
    rc = L.phg_laplace_calc2_noalloc(ops._h, C.c_void_p(out.data_ptr()), C.c_void_p(dF.data_ptr()),
                                     C.c_void_p(s.cuda_stream))
    assert rc == 0, L.phg_last_error().decode()
    assert L.phg_ops_check(ops._h, C.c_void_p(s.cuda_stream)) == 0
    want = phelm.SphereLaplace(ops).calc2(F)
    got = out.cpu().numpy()
    assert np.linalg.norm(got - want) / np.linalg.norm(want) <= 1e-13
