"""A level read from the on-disk cache (mesh, operators, multigrid hierarchy)
gives the same device operators as a freshly built one: solves and steps are
bit-identical."""
import gc

import numpy as np
import pytest

from mke_gb300 import fields, phelm, serve

pytestmark = pytest.mark.gpu


def run(level):
    m = phelm.Mesh.sphere(level)
    lat, lon = m.latlon()
    ops = phelm.Operators(m, phelm.PHG_MIXED, tol=1e-12)
    x = phelm.SphereLaplace(ops).solve(serve.solve_inputs(lat, lon, 1, seed=2)[0])
    bv = phelm.BarVortex(ops, coriolis=np.sin(lat), tau=1e-3, sigma=1.6e-2, mu=8e-5, theta=0.5, picard_iters=3)
    u = bv.calc(fields.barvortex_initial(lat, lon, seed=3)[0])
    del bv, ops, m
    gc.collect()
    return x, u


def test_cached_level_bit_identical(tmp_path):
    phelm.cache_dir(None)
    ref = run(5)
    phelm.cache_dir(str(tmp_path))
    try:
        run(5)                                # builds and writes the file
        assert (tmp_path / "phelm_level5.cache").exists()
        got = run(5)                          # reads it back
    finally:
        phelm.cache_dir(None)
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
