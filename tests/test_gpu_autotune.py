"""Autotuner (phg_ops_autotune): every candidate launch shape is timed, a
shape that misses the tolerance is never chosen, and the tuned shapes give
the same answers -- bit for bit where a shape only redistributes whole rows
(the interleaved operator apply), within the solve tolerance where it
changes the grouping of a reduction (the solver's row blocks)."""
import numpy as np
import pytest

from mke_gb300 import fields, phelm

pytestmark = pytest.mark.gpu

CONF = dict(tau=1e-3, sigma=1.6e-2, mu=8e-5, theta=0.5, picard_iters=3)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


@pytest.fixture(autouse=True)
def clean_table():
    phelm.tune_clear()
    yield
    phelm.tune_clear()


@pytest.mark.parametrize("precision", [phelm.PHG_FP64, phelm.PHG_MIXED])
def test_autotune_single_state(precision):
    m = phelm.Mesh.sphere(4)
    lat, lon = m.latlon()
    ops = phelm.Operators(m, precision, tol=1e-12)
    bv = phelm.BarVortex(ops, coriolis=np.sin(lat), **CONF)
    u0 = fields.barvortex_initial(lat, lon, seed=3)[0]
    before = bv.calc(u0)
    rep = ops.autotune(1)
    assert rep.count("chose") == 3, rep
    for rpb in (128, 256, 512, 1024):
        assert f"rpb={rpb} " in rep
    t = phelm.tune_table()
    rs = m.inner_size
    keys = {(e["family"], e["bucket"]) for e in t if e["kind"] == "solve" and e["rows"] == rs}
    assert {(1, 0), (1, 3), (2, 0)} <= keys
    after = bv.calc(u0)
    assert rel(after, before) <= 1e-9


def test_autotune_ensemble_mixed_lockstep_and_spmm():
    torch = pytest.importorskip("torch")
    m = phelm.Mesh.sphere(4)
    lat, lon = m.latlon()
    ops = phelm.Operators(m, phelm.PHG_MIXED, tol=1e-12)
    # the interleaved apply before tuning
    x = torch.randn((m.inner_size, 32), dtype=torch.float32, device="cuda")
    y0 = torch.empty_like(x)
    ops.mult32("lapl", x, y0)
    U0 = np.stack([fields.barvortex_initial(lat, lon, seed=10 + k)[0] for k in range(32)])
    bv = phelm.BarVortex(ops, coriolis=np.sin(lat), **CONF)
    before = bv.calc_batch(U0)
    rep = ops.autotune(32)
    assert "path=1" in rep            # the lockstep path was a candidate
    assert "threads_per_row=" in rep  # and the operator-apply widths
    spmm = [e for e in phelm.tune_table() if e["kind"] == "spmm"]
    assert len(spmm) == 1 and spmm[0]["rows"] == m.inner_size
    y1 = torch.empty_like(x)
    ops.mult32("lapl", x, y1)
    torch.cuda.synchronize()
    assert torch.equal(y0, y1)
    after = bv.calc_batch(U0)
    assert rel(after, before) <= 1e-9


def test_tuned_table_survives_save_load(tmp_path):
    m = phelm.Mesh.sphere(3)
    ops = phelm.Operators(m, phelm.PHG_MIXED, tol=1e-12)
    ops.autotune(4)
    t = phelm.tune_table()
    f = tmp_path / "tune.txt"
    phelm.tune_save(str(f))
    phelm.tune_clear()
    assert phelm.tune_load(str(f)) == len(t)
    assert sorted(map(str, phelm.tune_table())) == sorted(map(str, t))
