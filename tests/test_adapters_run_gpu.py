"""The C++ adapters of include/ccd_gb300_reference.hpp, run.

tests/adapter_run.cpp drives them as a reference program would: the CTCD
forwarders on the known answers of example/testCTCD.cpp, then
GpuKDOPBroadPhase, GpuAABBBroadPhase (with and without fixed vertices) and
GpuCTCDNarrowPhase on the reference's example meshes, through
libccd_gb300.so.  It is built against tests/adapter_standins/, which declare
the five reference headers the adapters include (the reference tree itself is
not needed), and the project's Eigen subset.  Its output must equal the
golden fixtures made from the reference: hits and contact times of the known
answers, the candidate sets' digests and the colliding sets' digest.
"""
import hashlib
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TOL = 1e-12


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode())
        h.update(str(a.shape).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def _build(tmp_path):
    from collisiondetection_gb300 import build as B

    lib = B.build_library()
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "adapter_run")
    cmd = [cxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror",
           "-I" + os.path.join(ROOT, "tests", "adapter_standins"),
           "-I" + os.path.join(ROOT, "collisiondetection_gb300", "eigen_subset"),
           "-I" + os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "adapter_run.cpp"),
           "-L" + os.path.dirname(lib), "-lccd_gb300", "-Wl,-rpath," + os.path.dirname(lib), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_adapters_run_against_golden(tmp_path, golden_dir):
    exe = _build(tmp_path)
    kat = json.load(open(os.path.join(golden_dir, "kat_testctcd.json")))
    meta = json.load(open(os.path.join(golden_dir, "meshes.json")))
    arrays = np.load(os.path.join(golden_dir, "meshes.npz"))
    names = ["test12", "prob3", "spheres"]

    lines = [f"kat {len(kat)}"]
    for c in kat:
        pts = " ".join(float(x).hex() for p in c["points"] for x in p)
        lines.append(f"{c['kind']} {float(c['eta']).hex()} {pts}")
    for name in names:
        qs = np.asarray(arrays[f"{name}_qstart"], np.float64).reshape(-1)
        qe = np.asarray(arrays[f"{name}_qend"], np.float64).reshape(-1)
        f = np.asarray(arrays[f"{name}_faces"]).reshape(-1)
        fixed = np.nonzero(np.asarray(arrays[f"{name}_fixed"]).reshape(-1))[0]
        lines.append(f"mesh {name} {qs.size // 3} {f.size // 3} {float(meta[name]['eta']).hex()} {fixed.size}")
        lines.append(" ".join(x.hex() for x in qs.tolist()))
        lines.append(" ".join(x.hex() for x in qe.tolist()))
        lines.append(" ".join(str(int(x)) for x in f))
        lines.append(" ".join(str(int(x)) for x in fixed))
    inp = tmp_path / "input.txt"
    inp.write_text("\n".join(lines) + "\n")
    r = subprocess.run([exe, str(inp)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr

    kat_out, cand, counts, hits = {}, {}, {}, {}
    for line in r.stdout.splitlines():
        w = line.split()
        if w[0] == "kat":
            kat_out[int(w[1])] = (int(w[2]), float.fromhex(w[3]))
        elif w[0] == "cand":
            cand.setdefault((w[1], w[2], w[3]), []).append([int(x) for x in w[4:8]])
        elif w[0] == "count":
            counts[(w[1], w[2])] = (int(w[3]), int(w[4]))
        elif w[0] == "hit":
            hits.setdefault((w[1], w[2]), set()).add(tuple(int(x) for x in w[3:7]))

    assert sorted(kat_out) == list(range(len(kat)))
    for i, c in enumerate(kat):
        h, t = kat_out[i]
        assert h == c["hit"] == 1
        assert abs(t - c["t"]) <= TOL * abs(c["t"])

    for name in names:
        for label in ("kdop", "aabb", "kdop_fixed", "aabb_fixed"):
            want = meta[name][label]
            vf = np.array(cand.get((name, label, "vf"), []), np.int32).reshape(-1, 4)
            ee = np.array(cand.get((name, label, "ee"), []), np.int32).reshape(-1, 4)
            assert counts[(name, label)] == (want["n_vf"], want["n_ee"]) == (vf.shape[0], ee.shape[0])
            assert digest(vf, ee) == want["digest"], (name, label)
        vf = np.array(cand.get((name, "kdop", "vf"), []), np.int32).reshape(-1, 4)
        ee = np.array(cand.get((name, "kdop", "ee"), []), np.int32).reshape(-1, 4)
        hv, he = hits.get((name, "vf"), set()), hits.get((name, "ee"), set())
        vf_hit = np.array([tuple(s) in hv for s in vf.tolist()], np.uint8)
        ee_hit = np.array([tuple(s) in he for s in ee.tolist()], np.uint8)
        assert (int(vf_hit.sum()), int(ee_hit.sum())) == (meta[name]["narrow"]["n_vf_hit"],
                                                          meta[name]["narrow"]["n_ee_hit"])
        assert digest(vf_hit, ee_hit) == meta[name]["narrow"]["digest"], name
