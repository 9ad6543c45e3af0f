"""The autotuner's shape table on the host: text form, save / load round
trip, files from another device model, malformed files (no GPU needed)."""
import pytest

from mke_gb300 import phelm


@pytest.fixture(autouse=True)
def clean_table():
    phelm.tune_clear()
    yield
    phelm.tune_clear()


def header(tmp_path):
    p = tmp_path / "empty.txt"
    phelm.tune_save(str(p))
    return p.read_text().splitlines()[0]


def test_save_load_round_trip(tmp_path):
    assert phelm.tune_table() == []
    f = tmp_path / "t.txt"
    f.write_text(header(tmp_path) + "\nsolve 1 10241 1 3 512 0\nsolve 2 10241 0 0 128 -1\nspmm 10241 5 4\n")
    assert phelm.tune_load(str(f)) == 3
    t = phelm.tune_table()
    assert dict(kind="solve", family=1, rows=10241, precision=1, bucket=3, rows_per_block=512, path=0) in t
    assert dict(kind="solve", family=2, rows=10241, precision=0, bucket=0, rows_per_block=128, path=-1) in t
    assert dict(kind="spmm", rows=10241, bucket=5, threads_per_row=4) in t
    g = tmp_path / "again.txt"
    phelm.tune_save(str(g))
    phelm.tune_clear()
    assert phelm.tune_table() == []
    assert phelm.tune_load(str(g)) == 3
    assert sorted(map(str, phelm.tune_table())) == sorted(map(str, t))


def test_other_device_model_is_ignored(tmp_path):
    f = tmp_path / "other.txt"
    f.write_text("phelm-gb300-tune 1 Some_Other_GPU_sm80\nsolve 1 642 1 0 128 0\n")
    assert phelm.tune_load(str(f)) == 0
    assert phelm.tune_table() == []


@pytest.mark.parametrize("body", ["solve 1 642 1 0\n", "spmm 642 2 3\n", "solve 1 642 1 0 128 7\n", "bogus 1\n"])
def test_malformed_files_are_rejected(tmp_path, body):
    f = tmp_path / "bad.txt"
    f.write_text(header(tmp_path) + "\n" + body)
    with pytest.raises(phelm.PhgError):
        phelm.tune_load(str(f))


def test_missing_file(tmp_path):
    with pytest.raises(phelm.PhgError):
        phelm.tune_load(str(tmp_path / "nope.txt"))
