"""Build libphelm_gb300.so in-tree (mke_gb300/_lib/).

Host C++ (mesh, assembly) is compiled by g++, the CUDA files by nvcc for
sm_103a only; the files compile in parallel and link with nvcc.  The kernels
file that must round like the CPU reference is compiled with -fmad=false;
host code uses -ffp-contract=off for the same reason.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libphelm_gb300.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-fopenmp", "-std=c++17"]

UNITS = [
    ("phg_mesh.cpp", "host", []),
    ("phg_assemble.cpp", "host", []),
    ("phg_cache.cpp", "host", []),
    ("phg_kernels.cu", "cuda", ["-fmad=false"]),
    ("phg_gmres.cu", "cuda", []),
    ("phg_capi.cu", "cuda", []),
    ("phg_serve.cu", "cuda", []),
    ("phg_tune.cu", "cuda", []),
    ("phg_jacquad.cu", "cuda", []),
]


def _sources():
    return [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".cu", ".cuh", ".cpp", ".hpp"))] + [
        os.path.join(os.path.dirname(HERE), "include", "phelm_gb300.h")]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(s) > t for s in _sources())


def _compile(unit):
    name, kind, extra = unit
    src = os.path.join(SRC, name)
    obj = os.path.join(OUT, name + ".o")
    if kind == "host":
        cmd = ["g++", *HOST, "-c", src, "-o", obj]
    else:
        cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", ",".join(HOST[:4] + ["-fopenmp"]),
               *extra, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if sources changed) and return the library path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(_compile, UNITS))
    tmp = LIB + ".tmp"
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fopenmp", "-lgomp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
