"""The analytic fields of tests/manufactured.py checked by finite differences
(CPU): the Laplace test field's Laplacian, the Jacobian pair's exact
Jacobian and the manufactured barotropic forcing satisfy their equations at
random points, so the GPU accuracy tests that use them check the library,
not a derivation slip."""
import numpy as np

import manufactured as mf

H = 1e-4


def lap_fd(f, phi, lam):
    fpp = (f(phi + H, lam) - 2 * f(phi, lam) + f(phi - H, lam)) / H ** 2
    fp = (f(phi + H, lam) - f(phi - H, lam)) / (2 * H)
    fll = (f(phi, lam + H) - 2 * f(phi, lam) + f(phi, lam - H)) / H ** 2
    return fpp - np.tan(phi) * fp + fll / np.cos(phi) ** 2


def jac_fd(u, v, phi, lam):
    d = lambda f, a, b: ((f(phi + a, lam + b) - f(phi - a, lam - b)) / (2 * H))  # noqa: E731
    return (d(u, 0, H) * d(v, H, 0) - d(u, H, 0) * d(v, 0, H)) / np.cos(phi)


def points(n=200, seed=0):
    rng = np.random.default_rng(seed)
    return rng.uniform(-1.4, 1.4, n), rng.uniform(-np.pi, np.pi, n)


def test_laplace_field():
    phi, lam = points()
    ex = mf.slaplace_lapl(phi, lam)
    assert np.max(np.abs(lap_fd(mf.slaplace_u, phi, lam) - ex)) <= 1e-5 * np.max(np.abs(ex))


def test_jacobian_pair():
    phi, lam = points()
    ex = mf.jac_exact(phi, lam)
    assert np.max(np.abs(jac_fd(mf.jac_f1, mf.jac_f2, phi, lam) - ex)) <= 1e-6 * np.max(np.abs(ex))


def test_barvortex_forcing():
    phi, lam = points()
    sigma, mu = 1.6e-2, 8e-5
    for t in (0.0, 0.37):
        psi = lambda p, l: mf.bv_psi(p, l, t)  # noqa: E731
        om = lambda p, l: mf.bv_omega(p, l, t)  # noqa: E731
        # omega is the Laplacian of psi
        assert np.max(np.abs(lap_fd(psi, phi, lam) - om(phi, lam))) <= 1e-5
        dt = (mf.bv_omega(phi, lam, t + H) - mf.bv_omega(phi, lam, t - H)) / (2 * H)
        lhs = dt + jac_fd(psi, om, phi, lam) + sigma * om(phi, lam) - mu * lap_fd(om, phi, lam)
        f = mf.bv_forcing(phi, lam, t, sigma, mu)
        assert np.max(np.abs(lhs - f)) <= 1e-5 * np.max(np.abs(f))
