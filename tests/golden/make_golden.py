"""Generate the golden fixtures from the reference's own sources.

Builds ``oracle/_ref`` (the reference's src/, examples/ and utils/ compiled
against the project-written linal shim, see oracle/Makefile), generates the
meshes with the reference's mesh generator, feeds seeded fields from
``mke_gb300.fields`` to ``oracle/_ref/ref_driver`` and stores what the
reference computed under tests/golden/.  Run it in a container that has the
reference tree (default /root/reference):

    python tests/golden/make_golden.py [--ref /root/reference] [--traj]

``--traj`` also integrates the level-6 barotropic trajectory (100 steps,
3 Picard iterations) -- a few minutes of CPU.
"""
from __future__ import annotations

import argparse
import hashlib
import shutil
import os
import subprocess
import sys
import tempfile

import numpy as np

# The reference fills a mutable per-triangle basis cache inside OpenMP loops
# (src/mesh.h:193, src/mesh.cpp:533-561); one thread avoids that race.
os.environ["OMP_NUM_THREADS"] = "1"

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
from mke_gb300 import fields  # noqa: E402

OPS = ["idt", "lapl", "bnd1", "bnd2", "bnd3", "jidt", "d1", "d2", "d1c", "d2c",
       "d1b", "d2b", "d1cb", "d2cb", "norm"]
MESH = ["xyz", "uv", "tri", "tz", "bnd", "inner", "outer", "p2io", "adj_ptr", "adj"]


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def run_level(ref_bin, level, work, bv_steps=0, bc_steps=0, seed=1234, extra=()):
    mesh_txt = os.path.join(work, f"ss{level}.txt")
    with open(mesh_txt, "w") as f:
        subprocess.run([os.path.join(ref_bin, "mke_mesh_sphere"), "--type", "full", "--coord", "local",
                        "--iter", str(level)], stdout=f, check=True)
    out = os.path.join(work, f"L{level}")
    os.makedirs(out, exist_ok=True)
    shutil.copyfile(mesh_txt, os.path.join(out, "mesh_text.txt"))
    # first pass: mesh only, to learn the coordinates for the inputs
    subprocess.run([os.path.join(ref_bin, "ref_driver"), mesh_txt, out], check=True,
                   stderr=subprocess.DEVNULL)
    uv = np.load(os.path.join(out, "mesh_uv.npy")).reshape(-1, 4, 2)
    bnd = np.load(os.path.join(out, "mesh_bnd.npy"))
    lat, lon = uv[:, 0, 0], uv[:, 0, 1]
    rng = np.random.default_rng(seed + level)
    u = fields.sh_field(fields.random_coeffs(rng, 1, 6), lat, lon)
    v = fields.sh_field(fields.random_coeffs(rng, 1, 6), lat, lon)
    np.save(os.path.join(out, "in_u.npy"), u)
    np.save(os.path.join(out, "in_v.npy"), v)
    np.save(os.path.join(out, "in_bnd.npy"), u[bnd == 1].copy())
    args = [os.path.join(ref_bin, "ref_driver"), mesh_txt, out,
            f"bv_steps={bv_steps}", f"bc_steps={bc_steps}", "bv_iters=3", "bc_iters=3", "bv_lin=1", "bc_lin=1",
            "bv_bf=1", *extra]
    subprocess.run(args, check=True, stderr=subprocess.DEVNULL)
    return out


def load_dir(d):
    r = {}
    for f in os.listdir(d):
        if f.endswith(".npy"):
            r[f[:-4]] = np.load(os.path.join(d, f))
        elif f.endswith(".txt"):   # text outputs: their SHA-256 (and without the first line: the
            data = open(os.path.join(d, f), "rb").read()   # generator's "#cmd:" line names its path)
            r["out_text_sha256_" + f[:-4]] = np.array(hashlib.sha256(data).hexdigest())
            r["out_text_sha256_" + f[:-4] + "_body"] = np.array(hashlib.sha256(data.split(b"\n", 1)[1]).hexdigest())
    return r


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--traj", action="store_true")
    a = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), f"REF={a.ref}", "ref"], check=True)
    ref_bin = os.path.join(REPO, "oracle", "_ref")
    with tempfile.TemporaryDirectory() as work:
        # levels 1-3: everything the reference computes, stored in full
        for level, bvs, bcs in ((1, 2, 1), (2, 2, 1), (3, 2, 1)):
            d = load_dir(run_level(ref_bin, level, work, bv_steps=bvs, bc_steps=bcs))
            keep = {k: v for k, v in d.items()}
            np.savez_compressed(os.path.join(HERE, f"ref_L{level}.npz"), **keep)
            print("level", level, "arrays", len(keep))
        # levels 4-5: mesh + operator digests and operator outputs
        for level in (4, 5):
            d = load_dir(run_level(ref_bin, level, work, bv_steps=1 if level == 4 else 0))
            keep = {k: v for k, v in d.items() if k.startswith(("in_", "out_"))}
            keep["digest_mesh"] = np.array(digest(*[d["mesh_" + k] for k in MESH]))
            for k in ("tri", "tz", "inner", "p2io"):
                keep["mesh_" + k] = d["mesh_" + k]
            for op in OPS:
                keep["digest_" + op] = np.array(digest(d[op + "_ptr"], d[op + "_col"], d[op + "_val"]))
                keep["pattern_" + op] = np.array(digest(d[op + "_ptr"], d[op + "_col"]))
            np.savez_compressed(os.path.join(HERE, f"ref_L{level}.npz"), **keep)
            print("level", level, "arrays", len(keep))
        # the reference's accuracy checks on the analytic fields of tests/manufactured.py
        pins = {}
        for level in (3, 4, 5):
            mesh_txt = os.path.join(work, f"ss{level}.txt")
            out = os.path.join(work, f"pins{level}")
            os.makedirs(out, exist_ok=True)
            subprocess.run([os.path.join(ref_bin, "ref_driver"), mesh_txt, out, f"pins={1 if level == 3 else 2}"],
                           check=True, stderr=subprocess.DEVNULL)
            for k in ("slaplace", "jacobian", "barvortex"):
                f = os.path.join(out, f"out_pin_{k}.npy")
                if os.path.exists(f):
                    pins[f"{k}_L{level}"] = np.load(f)
        np.savez_compressed(os.path.join(HERE, "ref_pins.npz"), **pins)
        print("accuracy pins", {k: v.tolist() for k, v in pins.items()})
        if a.traj:
            level = 6
            mesh_txt = os.path.join(work, "ss6.txt")
            with open(mesh_txt, "w") as f:
                subprocess.run([os.path.join(ref_bin, "mke_mesh_sphere"), "--type", "full", "--coord",
                                "local", "--iter", "6"], stdout=f, check=True)
            out = os.path.join(work, "L6")
            os.makedirs(out, exist_ok=True)
            subprocess.run([os.path.join(ref_bin, "ref_driver"), mesh_txt, out], check=True,
                           stderr=subprocess.DEVNULL)
            uv = np.load(os.path.join(out, "mesh_uv.npy")).reshape(-1, 4, 2)
            psi0, _ = fields.barvortex_initial(uv[:, 0, 0], uv[:, 0, 1], seed=2024)
            np.save(os.path.join(out, "in_u.npy"), psi0)
            subprocess.run([os.path.join(ref_bin, "ref_driver"), mesh_txt, out, "bv_steps=100",
                            "bv_iters=3"], check=True, stderr=subprocess.DEVNULL)
            d = load_dir(out)
            keep = {"in_u": d["in_u"], "out_bv_step1": d["out_bv_step1"], "out_bv_final": d["out_bv_final"],
                    "digest_mesh": np.array(digest(*[d["mesh_" + k] for k in MESH]))}
            for op in OPS:
                keep["pattern_" + op] = np.array(digest(d[op + "_ptr"], d[op + "_col"]))
            np.savez_compressed(os.path.join(HERE, "ref_L6_barvortex100.npz"), **keep)
            print("level 6 trajectory stored")


if __name__ == "__main__":
    main()
