"""The drop-in C++ shim: pRRTC::solve<Robot> with the reference's signature,
compiled against stand-in reference types (and against the reference's own
headers where they are present) and linked to the library."""
import subprocess

import numpy as np
import pytest

from conftest import REFERENCE, ROOT


def build_driver(tmp_path, reference_headers=False):
    import prrtc_gb300.build as b
    lib = b.build()
    exe = tmp_path / ("solve_ref" if reference_headers else "solve_standin")
    cmd = ["g++", "-std=c++17", "-O1", f"-I{ROOT / 'include'}", f"-I{ROOT / 'tests/cpp'}",
           str(ROOT / "tests/cpp/solve_compat.cpp"), "-o", str(exe), f"-L{lib.parent}", "-lprrtc_gb300",
           f"-Wl,-rpath,{lib.parent}"]
    if reference_headers:
        cmd[1:1] = ["-DUSE_REFERENCE_HEADERS", "-DmemoryClockRate=memoryBusWidth", f"-I{REFERENCE}",
                    f"-I{REFERENCE / 'src'}", "-I/usr/local/cuda/include", "-w"]
        cmd += ["-L/usr/local/cuda/lib64", "-lcudart"]
    subprocess.run(cmd, check=True)
    return exe


def test_shim_compiles_and_links_with_standins(tmp_path):
    assert build_driver(tmp_path).exists()


@pytest.mark.skipif(not (REFERENCE / "src/planning/Planners.hh").exists(), reason="reference checkout absent")
def test_shim_compiles_against_reference_headers(tmp_path):
    assert build_driver(tmp_path, reference_headers=True).exists()


@pytest.mark.gpu
def test_shim_solves_and_path_revalidates(tmp_path, oracle):
    from prrtc_gb300 import scenes
    exe = build_driver(tmp_path)
    q = scenes.make_query("panda", "tabletop", 7)
    lines = [str(len(q.env.spheres))] + [" ".join(map(repr, map(float, r))) for r in q.env.spheres]
    lines += [str(len(q.env.cuboids))] + [" ".join(map(repr, map(float, r))) for r in q.env.cuboids]
    lines += [" ".join(map(repr, map(float, q.start))), " ".join(map(repr, map(float, q.goal)))]
    out = subprocess.run([str(exe)], input="\n".join(lines), capture_output=True, text=True, check=True).stdout.split("\n")
    solved, cost, rows = out[0].split()
    assert solved == "1"
    path = np.array([[float(v) for v in l.split()] for l in out[1:1 + int(rows)]], np.float32)
    np.testing.assert_array_equal(path[0], q.goal)
    np.testing.assert_array_equal(path[-1], q.start)
    assert oracle.check_edges("panda", q.env, path[:-1], path[1:], 32).all()
