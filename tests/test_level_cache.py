"""The host-side level cache (phg_cache_dir): a generated level is written to
disk once with its mesh, operators and multigrid hierarchy, read back byte for
byte by later generations, and a damaged file is rejected and rebuilt.  No GPU
needed (mesh arrays and assembled operators are host data)."""
import gc
import os
import struct

import numpy as np
import pytest

from mke_gb300 import phelm

OPS = ["idt", "lapl", "jidt", "d1", "d2", "d1c", "d2c", "bnd2", "bnd3", "d1b", "d2b", "d1cb", "d2cb", "norm"]


def snapshot(level):
    m = phelm.Mesh.sphere(level)
    out = {k: v.copy() for k, v in m.arrays().items()}
    for name in OPS:
        p, c, v = m.csr(name)
        out[name] = (p.copy(), c.copy(), v.copy())
    del m
    gc.collect()
    return out


def same(a, b):
    for k in a:
        if isinstance(a[k], tuple):
            if not all(np.array_equal(x, y) for x, y in zip(a[k], b[k])):
                return False
        elif not np.array_equal(a[k], b[k], equal_nan=True):
            return False
    return True


def fnv1a(data: bytes) -> int:
    h = 1469598103934665603
    for byte in data:
        h = ((h ^ byte) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


@pytest.fixture
def cache(tmp_path):
    phelm.cache_dir(str(tmp_path))
    yield tmp_path
    phelm.cache_dir(None)
    gc.collect()


def test_written_then_read_back_identical(cache):
    phelm.cache_dir(None)
    fresh = snapshot(3)
    phelm.cache_dir(str(cache))
    first = snapshot(3)                      # generated, assembled and saved
    path = cache / "phelm_level3.cache"
    assert path.exists() and path.read_bytes()[:8] == b"PHGLVL01"
    second = snapshot(3)                     # read from the file
    assert same(fresh, first) and same(fresh, second)


def test_data_come_from_the_file(cache):
    snapshot(3)
    path = cache / "phelm_level3.cache"
    raw = bytearray(path.read_bytes())
    # payload: 6 int32 mesh scalars, then xyz as uint64 count + doubles
    off = 12 + 24 + 8
    x0 = struct.unpack_from("<d", raw, off)[0]
    struct.pack_into("<d", raw, off, x0 + 1.0)
    struct.pack_into("<Q", raw, len(raw) - 8, fnv1a(bytes(raw[12:-8])))
    path.write_bytes(bytes(raw))
    m = phelm.Mesh.sphere(3)
    assert m.arrays()["xyz"][0] == x0 + 1.0   # the edited (but well-formed) file was used
    del m
    gc.collect()


@pytest.mark.parametrize("damage", ["flip", "truncate", "level", "magic"])
def test_damaged_file_is_rebuilt(cache, damage):
    phelm.cache_dir(None)
    fresh = snapshot(3)
    phelm.cache_dir(str(cache))
    snapshot(3)
    path = cache / "phelm_level3.cache"
    raw = bytearray(path.read_bytes())
    if damage == "flip":
        raw[len(raw) // 2] ^= 0x40
    elif damage == "truncate":
        raw = raw[: len(raw) // 3]
    elif damage == "level":
        struct.pack_into("<i", raw, 8, 4)
    else:
        raw[0:8] = b"NOTACASH"
    path.write_bytes(bytes(raw))
    assert same(fresh, snapshot(3))           # rebuilt from scratch
    assert path.read_bytes()[:8] == b"PHGLVL01"
    assert same(fresh, snapshot(3))           # and the rewritten file reads back


MESH_VECS = [("xyz", 8), ("uv", 8), ("tri", 4), ("tz", 4), ("bnd", 4), ("inner", 4), ("outer", 4), ("p2io", 4),
             ("adj_ptr", 4), ("adj", 4), ("orig", 4), ("par_a", 4), ("par_b", 4), ("raw_xyz", 8)]


def layout(raw):
    """Byte offsets of the first mesh record's arrays and of the first
    operator record (file: magic, int32 level, then the payload)."""
    off = 12 + 24                      # level, V, T, rs, os, nz
    where = {}
    for name, size in MESH_VECS:
        n = struct.unpack_from("<Q", raw, off)[0]
        where[name] = (off + 8, n)
        off += 8 + n * size
    where["first_op"] = off            # int32 n, int32 m, then ptr / col / val
    return where


@pytest.mark.parametrize("edit", ["adjacency", "triangle", "orig", "operator_shape"])
def test_inconsistent_file_is_rebuilt(cache, edit):
    """A file with a valid checksum whose contents do not fit together (an
    index the assembly or the kernels would follow out of range) is rejected
    like a damaged one."""
    phelm.cache_dir(None)
    fresh = snapshot(3)
    phelm.cache_dir(str(cache))
    snapshot(3)
    path = cache / "phelm_level3.cache"
    original = path.read_bytes()
    raw = bytearray(original)
    w = layout(raw)
    V = struct.unpack_from("<i", raw, 16)[0]
    if edit == "adjacency":            # point 0's first triangle swapped for one not through it
        off, n = w["adj"]
        struct.pack_into("<i", raw, off, struct.unpack_from("<i", raw, off + 4 * (n - 1))[0])
    elif edit == "triangle":
        struct.pack_into("<i", raw, w["tri"][0], V)
    elif edit == "orig":               # no longer a permutation
        off, _ = w["orig"]
        struct.pack_into("<i", raw, off, struct.unpack_from("<i", raw, off + 4)[0])
    else:                              # idt: one column more than the inner points
        off = w["first_op"] + 4
        struct.pack_into("<i", raw, off, struct.unpack_from("<i", raw, off)[0] + 1)
    struct.pack_into("<Q", raw, len(raw) - 8, fnv1a(bytes(raw[12:-8])))
    path.write_bytes(bytes(raw))
    assert same(fresh, snapshot(3))           # rebuilt from scratch
    assert path.read_bytes() == original      # the rejected file was rewritten
    assert same(fresh, snapshot(3))


WRITER = r"""
import sys
sys.path.insert(0, sys.argv[1])
from mke_gb300 import phelm
phelm.cache_dir(sys.argv[2])
m = phelm.Mesh.sphere(4)
print(m.size)
"""


def test_processes_building_one_level_at_once(tmp_path):
    """Processes that build the same level into one cache directory at the
    same time each write a temporary file of their own and rename it: one
    valid file remains, no temporary is left behind."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    procs = [subprocess.Popen([sys.executable, "-c", WRITER, root, str(tmp_path)], stdout=subprocess.PIPE,
                              stderr=subprocess.PIPE, text=True) for _ in range(4)]
    for p in procs:
        out, err = p.communicate(timeout=300)
        assert p.returncode == 0, err[-2000:]
        assert out.strip() == "2562"
    assert sorted(f.name for f in tmp_path.iterdir()) == ["phelm_level4.cache"]
    phelm.cache_dir(None)
    fresh = snapshot(4)
    phelm.cache_dir(str(tmp_path))
    try:
        inode = (tmp_path / "phelm_level4.cache").stat().st_ino
        assert same(fresh, snapshot(4))                            # read from the file
        assert (tmp_path / "phelm_level4.cache").stat().st_ino == inode   # accepted: a rewrite renames a new file
    finally:
        phelm.cache_dir(None)
        gc.collect()


def test_unwritable_directory_is_not_an_error(tmp_path):
    missing = tmp_path / "does" / "not" / "exist"
    phelm.cache_dir(str(missing))
    try:
        m = phelm.Mesh.sphere(2)
        assert m.size == 162
        del m
    finally:
        phelm.cache_dir(None)
        gc.collect()


def test_handles_of_one_level_share_data():
    a = phelm.Mesh.sphere(3)
    b = phelm.Mesh.sphere(3)
    pa, _, _ = a.csr("lapl")
    pb, _, _ = b.csr("lapl")
    assert np.array_equal(pa, pb)
    del a
    gc.collect()
    assert b.csr("lapl")[0].size == pb.size  # b's data survives a's destruction


def test_live_level_written_when_directory_set_later(tmp_path):
    phelm.cache_dir(None)
    keep = phelm.Mesh.sphere(3)              # alive while the directory is set
    phelm.cache_dir(str(tmp_path))
    try:
        other = phelm.Mesh.sphere(3)         # shares keep's data and writes the file
        assert (tmp_path / "phelm_level3.cache").exists()
        del other
    finally:
        phelm.cache_dir(None)
    del keep
    gc.collect()


def test_concurrent_generation():
    """Different levels build concurrently and one level once; every handle
    equals a serially built one (ctypes releases the GIL during the calls)."""
    import threading
    phelm.cache_dir(None)
    ref = {lv: snapshot(lv) for lv in (2, 3, 4)}
    got = {}
    errors = []

    def work(lv, k):
        try:
            m = phelm.Mesh.sphere(lv)
            p, c, v = m.csr("lapl")
            got[(lv, k)] = (m.arrays()["xyz"].copy(), p.copy(), c.copy(), v.copy())
        except Exception as e:   # reported below
            errors.append(repr(e))

    threads = [threading.Thread(target=work, args=(lv, k)) for lv in (2, 3, 4) for k in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(120)
    assert not errors, errors
    for (lv, k), (xyz, p, c, v) in got.items():
        assert np.array_equal(xyz, ref[lv]["xyz"])
        assert all(np.array_equal(a, b) for a, b in zip((p, c, v), ref[lv]["lapl"]))
    gc.collect()
