"""The host code and the CPU oracle under AddressSanitizer and
UndefinedBehaviorSanitizer (no GPU): tests/sanitize/host_driver.cpp runs the
library's mesh generation, text I/O and assembly at levels 1-4, and the level
cache reader and the mesh text parser on damaged files,
tests/sanitize/oracle_driver.c the oracle's solves and steps at levels 2-3.
Each is compiled here with -fsanitize=address,undefined and must exit 0 with
no sanitizer report."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SAN = ["-fsanitize=address,undefined", "-fno-omit-frame-pointer", "-fno-sanitize-recover=all", "-O1", "-g"]
ENV = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:halt_on_error=1:abort_on_error=0",
           UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1", OMP_NUM_THREADS="2")


def sanitizers_available(tmp_path):
    if not shutil.which("g++") or not shutil.which("gcc"):
        return False
    src = tmp_path / "probe.cpp"
    src.write_text("int main() { return 0; }\n")
    r = subprocess.run(["g++", *SAN, str(src), "-o", str(tmp_path / "probe")], capture_output=True)
    return r.returncode == 0


def run_checked(cmd, exe, *args):
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    p = subprocess.run([exe, *args], capture_output=True, text=True, env=ENV, timeout=900)
    report = p.stdout + p.stderr
    assert p.returncode == 0, report[-4000:]
    assert "runtime error" not in report and "AddressSanitizer" not in report, report[-4000:]
    return report


def test_host_code(tmp_path):
    if not sanitizers_available(tmp_path):
        pytest.skip("no sanitizer runtime")
    csrc = os.path.join(ROOT, "mke_gb300", "csrc")
    exe = str(tmp_path / "host_driver")
    cmd = ["g++", "-std=c++17", "-fopenmp", "-ffp-contract=off", *SAN, "-I", csrc,
           os.path.join(HERE, "sanitize", "host_driver.cpp"), os.path.join(csrc, "phg_mesh.cpp"),
           os.path.join(csrc, "phg_assemble.cpp"), os.path.join(csrc, "phg_cache.cpp"), "-o", exe]
    report = run_checked(cmd, exe, str(tmp_path))
    assert "host code clean" in report and "damaged files read" in report and "damaged mesh files read" in report


def test_oracle(tmp_path):
    if not sanitizers_available(tmp_path):
        pytest.skip("no sanitizer runtime")
    odir = os.path.join(ROOT, "oracle")
    srcs = [os.path.join(odir, f) for f in ("orc_linalg.c", "orc_mesh.c", "orc_assemble.c", "orc_model.c")]
    exe = str(tmp_path / "oracle_driver")
    cmd = ["gcc", "-std=gnu11", "-fopenmp", "-ffp-contract=off", *SAN, "-I", odir,
           os.path.join(HERE, "sanitize", "oracle_driver.c"), *srcs, "-lm", "-o", exe]
    assert "oracle clean" in run_checked(cmd, exe)
