"""The C++ facade shipped as include/phelm_gb300.hpp.

On the CPU: the header compiles against include/phelm_gb300.h (syntax and
types, no link), so the facade and the C ABI cannot drift apart.  On the GPU:
a small C++ program written the way a reference caller writes its code
(examples/test_barvortex.cpp, examples/test_slaplace.cpp) is compiled
against the facade, linked with libphelm_gb300.so and run; its results are
checked against the oracle.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")

DRIVER = r"""
#include "phelm_gb300.hpp"
#include <cmath>
#include <cstdio>
#include <vector>
using namespace phelm_gb300;

int main(int argc, char **argv) {
    const int level = 3;
    Mesh m(level);
    Operators ops(m, PHG_FP64);
    ops.set_solver(30, 1e-12, 20000);
    SphereLaplace<double> l(ops);
    SphereJacobian j(ops);
    SphereNorm<double> nrm(ops);
    std::vector<double> xyz(3 * m.size), uv(8 * m.size);
    phg_mesh_arrays(m.handle(), xyz.data(), uv.data(), nullptr, nullptr, nullptr);
    std::vector<double> u(m.size), v(m.size), cor(m.size), out(m.size), lap(m.size), jac(m.inner_size);
    for (int i = 0; i < m.size; ++i) {
        double phi = uv[8 * i], la = uv[8 * i + 1];
        u[i] = 0.1 * std::cos(phi) * std::cos(phi) * std::sin(2 * la) + 0.05 * std::sin(phi);
        v[i] = 0.2 * std::cos(phi) * std::cos(la);
        cor[i] = std::sin(phi);
    }
    l.calc1(&lap[0], &u[0], nullptr);
    j.calc2(&jac[0], &u[0], &v[0]);
    double n = nrm.norm(&u[0]);
    BarVortex bv(ops, barvortex_conf(1e-3, 1.6e-2, 8e-5, 1.0, 1.0, 0.5, 3), &cor[0]);
    bv.S_step(&out[0], &u[0]);
    FILE *f = fopen(argv[1], "wb");
    fwrite(&u[0], 8, m.size, f); fwrite(&v[0], 8, m.size, f);
    fwrite(&lap[0], 8, m.size, f); fwrite(&jac[0], 8, m.inner_size, f);
    fwrite(&n, 8, 1, f); fwrite(&out[0], 8, m.size, f);
    fclose(f);
    try { Mesh bad(0); return 3; } catch (const Error &e) { if (e.code != PHG_ERR_ARG) return 4; }
    return 0;
}
"""


def test_facade_compiles(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("no C++ compiler")
    src = tmp_path / "facade.cpp"
    src.write_text('#include "phelm_gb300.hpp"\nint main() { return 0; }\n')
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-I", INC, str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    drv = tmp_path / "driver.cpp"
    drv.write_text(DRIVER)
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-I", INC, str(drv)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_facade_program_runs(tmp_path):
    """A reference-style C++ caller through the facade: Laplace apply,
    Jacobian, norm and one barotropic step (S_step) at level 3 vs the oracle."""
    import pyoracle as po
    from mke_gb300 import build
    lib = build.build()
    drv = tmp_path / "driver.cpp"
    drv.write_text(DRIVER)
    exe = tmp_path / "driver"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", INC, str(drv), "-o", str(exe), lib,
                        "-Wl,-rpath," + os.path.dirname(lib)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    res = tmp_path / "out.bin"
    r = subprocess.run([str(exe), str(res)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stderr)
    o = po.Oracle(3)
    V, rs = o.V, o.rs
    d = np.fromfile(res, dtype=np.float64)
    u, v, lap, jac = d[:V], d[V:2 * V], d[2 * V:3 * V], d[3 * V:3 * V + rs]
    n, step = d[3 * V + rs], d[3 * V + rs + 1:]

    def rel(a, b):
        return np.linalg.norm(a - b) / np.linalg.norm(b)

    assert rel(lap, o.laplace_calc1(u, None)) <= 1e-13
    assert rel(jac, o.jacobian_calc2(u, v)) <= 1e-13
    assert abs(n - o.norm(u)) <= 1e-13 * o.norm(u)
    lat = o.mesh_arrays()["uv"].reshape(-1, 4, 2)[:, 0, 0]
    z = np.zeros(o.os)
    want = o.bv_step(o.barvortex(max_iter=3, coriolis=np.sin(lat)), u, z, z)
    assert rel(step, want) <= 1e-9
