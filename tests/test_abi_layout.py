"""The ctypes mirrors of the C ABI's structs (collisiondetection_gb300/_native.py)
against the header itself: a C program compiled with the host compiler
prints each struct's size and each field's offset, and they must equal
ctypes' layout, so a field added or moved on one side only fails here and
not as a silently misread result.  CPU only."""
import ctypes
import shutil
import subprocess

import pytest

import collisiondetection_gb300._native as N

PAIRS = [("ccd_batch_stats", N.BatchStats), ("ccd_batch_timings", N.BatchTimings),
         ("ccd_tune_result", N.TuneResult), ("ccd_fp64_peak_result", N.Fp64Peak),
         ("ccd_mesh_stats", N.MeshStats), ("ccd_velocity_filter_stats", N.VelocityFilterStats),
         ("ccd_request", N.Request), ("ccd_request_result", N.RequestResult)]


def test_ctypes_structs_match_the_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stddef.h>", "#include <stdio.h>", f'#include "{N.HEADER}"', "int main(void) {"]
    for cname, py in PAIRS:
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-o", str(exe), str(src)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        name, field, value = line.split()
        got[name, field] = int(value)
    for cname, py in PAIRS:
        assert got[cname, "size"] == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[cname, f] == getattr(py, f).offset, (cname, f)
