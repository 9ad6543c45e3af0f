"""The product library on the CPU: it loads, exports every declared entry
point, and its host-side mesh generator / loader / assembly reproduce the
reference exactly (golden fixtures from the reference's own sources)."""
import hashlib
import os
import re

import numpy as np
import pytest

from mke_gb300 import phelm

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OPS = ["idt", "lapl", "bnd2", "bnd3", "jidt", "d1", "d2", "d1c", "d2c", "d1b", "d2b", "d1cb", "d2cb", "norm"]


def header_symbols():
    txt = open(os.path.join(REPO, "include", "phelm_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(phg_[A-Za-z0-9_]+)\s*\(", txt)))


def test_exports_every_declared_symbol():
    L = phelm.lib()
    names = header_symbols()
    assert len(names) >= 25
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(phelm.SIGNATURES), set(names) ^ set(phelm.SIGNATURES)


def bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.int64)


@pytest.mark.parametrize("level", [1, 2, 3])
def test_mesh_and_operators_bitexact(level, golden):
    g = golden(f"ref_L{level}.npz")
    m = phelm.Mesh.sphere(level)
    a = m.arrays()
    for k in ("tri", "tz", "bnd"):
        assert np.array_equal(a[k], g["mesh_" + k]), k
    for k in ("xyz", "uv"):
        assert np.array_equal(bits(a[k]), bits(g["mesh_" + k])), k
    mp = m.maps()
    for k in ("inner", "outer", "p2io"):
        assert np.array_equal(mp[k], g["mesh_" + k]), k
    for op in OPS:
        p, c, v = m.csr(op)
        assert np.array_equal(p, g[op + "_ptr"]) and np.array_equal(c, g[op + "_col"]), op
        assert np.array_equal(v, g[op + "_val"]), op


@pytest.mark.parametrize("level", [4, 5])
def test_larger_levels_by_digest(level, golden):
    g = golden(f"ref_L{level}.npz")
    m = phelm.Mesh.sphere(level)
    a = m.arrays()
    for k in ("tri", "tz"):
        assert np.array_equal(a[k], g["mesh_" + k]), k
    for op in OPS:
        h = hashlib.sha256()
        for x in m.csr(op):
            h.update(np.ascontiguousarray(x).tobytes())
        assert h.hexdigest() == str(g["digest_" + op]), op


def write_reference_text(path, m):
    """The reference generator's text format (utils/icosahedron.cpp:268-457)."""
    a = m.arrays()
    xyz, uv = a["xyz"].reshape(-1, 3), a["uv"].reshape(-1, 4, 2)
    with open(path, "w") as f:
        f.write("#points:%d\n#triangles:%d\n" % (m.size, m.ntri))
        for k in range(4):
            f.write("#predef: zone %d stdsphere%d\n" % (k + 1, k + 1))
        for p in range(m.size):
            f.write("%.16f %.16f %.16f" % tuple(xyz[p]))
            for k in range(4):
                f.write(" ; %.16f %.16f " % tuple(uv[p, k]))
            f.write("\n")
        f.write("# triangles %d \n" % m.ntri)
        tri = a["tri"].reshape(-1, 3)
        for t in range(m.ntri):
            f.write("%d %d %d " % tuple(tri[t] + 1))
            if a["tz"][t] != 0:
                f.write(" ; %d " % (a["tz"][t] + 1))
            f.write("\n")
        f.write("# boundary \n")
        for p in np.nonzero(a["bnd"])[0]:
            f.write("%d \n" % (p + 1))


def test_load_text_roundtrip(tmp_path):
    m = phelm.Mesh.sphere(3)
    path = str(tmp_path / "ss3.txt")
    write_reference_text(path, m)
    m2 = phelm.Mesh.load(path)
    a, b = m.arrays(), m2.arrays()
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(m.csr("lapl")[2], m2.csr("lapl")[2])


def test_concurrent_text_loads(tmp_path):
    """Mesh files parse correctly when several threads load at once (ctypes
    releases the GIL during the call; the parser keeps no shared state)."""
    import threading
    m = phelm.Mesh.sphere(4)
    path = str(tmp_path / "ss4.txt")
    write_reference_text(path, m)
    want = m.arrays()
    bad = []

    def work():
        for _ in range(3):
            try:
                got = phelm.Mesh.load(path).arrays()
                if not all(np.array_equal(want[k], got[k], equal_nan=True) for k in want):
                    bad.append("arrays differ")
            except phelm.PhgError as e:
                bad.append(str(e))

    threads = [threading.Thread(target=work) for _ in range(8)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(300)
    assert not bad, bad[:3]


def test_errors():
    with pytest.raises(phelm.PhgError) as e:
        phelm.Mesh.sphere(0)
    assert e.value.code == 1
    with pytest.raises(phelm.PhgError) as e:
        phelm.Mesh.load("/nonexistent/mesh.txt")
    assert e.value.code == 5


HOST_OOM = r"""
import ctypes as C, resource, sys
sys.path.insert(0, sys.argv[1])
from mke_gb300 import phelm
L = phelm.lib()
vm = next(int(x.split()[1]) * 1024 for x in open("/proc/self/status") if x.startswith("VmSize:"))
resource.setrlimit(resource.RLIMIT_AS, (vm + 150 * 2**20, resource.RLIM_INFINITY))
h = C.c_void_p()
rc = L.phg_mesh_generate(9, C.byref(h))
print(rc, L.phg_last_error().decode())
print(L.phg_mesh_generate(2, C.byref(h)))
"""


def test_host_exception_becomes_status():
    """A C++ exception inside an entry point (here std::bad_alloc: a level-9 mesh
    under an address-space limit 150 MiB above the process's size) returns
    PHG_ERR_HOST instead of unwinding into the C caller, and the library stays
    usable.  One OpenMP thread, so that no thread creation meets the limit."""
    import subprocess
    import sys
    env = dict(os.environ, OMP_NUM_THREADS="1")
    p = subprocess.run([sys.executable, "-c", HOST_OOM, REPO], capture_output=True, text=True, env=env, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    first, second = p.stdout.strip().splitlines()[-2:]
    assert first == "7 host memory exhausted", first
    assert second == "0"


def test_no_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    m = phelm.Mesh.sphere(2)
    with pytest.raises(phelm.PhgError) as e:
        phelm.Operators(m)
    assert e.value.code == 2


@pytest.mark.parametrize("level", [1, 2, 3, 4, 5])
def test_text_outputs_match_reference(golden, level, tmp_path):
    """The mesh file (as mke_mesh_sphere writes it, utils/icosahedron.cpp:268-457)
    and print_function / print_inner_function (src/phelm.cpp:160-321) give the
    reference's bytes; the mesh file's first line is the generator's command
    line with its path, so it is compared from the second line on."""
    import hashlib
    g = golden(f"ref_L{level}.npz")
    m = phelm.Mesh.sphere(level)
    p = tmp_path / "mesh.txt"
    m.save(str(p))
    body = p.read_bytes().split(b"\n", 1)[1]
    assert hashlib.sha256(body).hexdigest() == str(g["out_text_sha256_mesh_text_body"])
    for inner, key in ((False, "print_function"), (True, "print_inner_function")):
        q = tmp_path / f"{key}.txt"
        m.print_function(str(q), g["in_u"], inner=inner)
        assert hashlib.sha256(q.read_bytes()).hexdigest() == str(g["out_text_sha256_" + key]), key
    # and the written file loads back into the same mesh
    m2 = phelm.Mesh.load(str(p))
    a, b = m.arrays(), m2.arrays()
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_state_checkpoint_round_trip(tmp_path):
    m = phelm.Mesh.sphere(3)
    rng = np.random.default_rng(5)
    u1, u2 = rng.standard_normal(m.size), rng.standard_normal(m.size)
    p = str(tmp_path / "state.bin")
    m.save_state(p, [u1, u2], t=0.25, step=250)
    (a, b), t, step = m.load_state(p, 2)
    assert np.array_equal(a, u1) and np.array_equal(b, u2) and t == 0.25 and step == 250
    with pytest.raises(phelm.PhgError):
        phelm.Mesh.sphere(4).load_state(p, 2)      # another mesh
    with pytest.raises(phelm.PhgError):
        m.load_state(p, 3)                         # another field count
