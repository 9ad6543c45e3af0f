"""Host side of the serving traces (no GPU): seeded, reproducible traces and
input pools with the configured shapes."""
import numpy as np

from mke_gb300 import fields, phelm, serve


def test_trace_is_seeded_and_sorted():
    a = serve.make_trace(n=2000, rate=2000.0, seed=7)
    b = serve.make_trace(n=2000, rate=2000.0, seed=7)
    assert a == b
    t = np.array([r[0] for r in a])
    assert np.all(np.diff(t) > 0)
    # Poisson arrivals at the requested mean rate
    assert abs(len(a) / t[-1] - 2000.0) < 200.0
    kinds = np.array([r[1] for r in a])
    assert abs((kinds == phelm.PHG_REQ_LAPLACE_SOLVE).mean() - 0.6) < 0.05
    levels = {r[2] for r in a}
    assert levels == {3, 4, 5, 6, 7}
    assert all(r[3] == (10 if r[1] == phelm.PHG_REQ_BARVORTEX else 1) for r in a)


def test_inputs_match_the_field_formulas():
    lat, lon = phelm.Mesh.sphere(3).latlon()
    F = serve.solve_inputs(lat, lon, 3, seed=1)
    assert F.shape == (3, lat.size)
    # a single mode reproduces real_sph_harm
    B, ls = serve.sh_basis(lat, lon, 4)
    Y = fields.real_sph_harm(4, lat, lon)
    assert np.allclose(B[ls.tolist().index(2.0)], Y[(2, -2)])
    psi = serve.barvortex_inputs(lat, lon, 2, seed=3)
    rh = fields.rossby_haurwitz4(lat, lon, 0.1) / -30.0
    # RH4 stream function plus a small (amplitude 1e-3 in vorticity) perturbation
    assert np.abs(psi - rh[None, :]).max() < 1e-3
    assert np.abs(psi - rh[None, :]).max() > 0
