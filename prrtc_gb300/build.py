"""Compile the library (sm_103a) in-tree: prrtc_gb300/libprrtc_gb300.so.

Each .cu under csrc/ is one nvcc job (the per-robot kernel files dominate);
jobs run in parallel and only out-of-date objects are rebuilt.  The build
holds an exclusive file lock (_build/.lock), so processes that start together
(one per GPU) build once and the others wait for it.
"""
from __future__ import annotations

import fcntl
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "libprrtc_gb300.so"
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
         f"-I{ROOT / 'include'}", f"-I{CSRC}"]
SOURCES = ["capi.cu", "planner.cu", "batch.cu", "noalloc.cu", "clearance.cu", "robot_sphere.cu", "robot_panda.cu", "robot_fetch.cu", "robot_baxter.cu"]


def _deps() -> float:
    newest = 0.0
    for p in list(CSRC.rglob("*.h")) + list(CSRC.rglob("*.cuh")) + list((ROOT / "include").rglob("*.h")):
        newest = max(newest, p.stat().st_mtime)
    return newest


def _compile(src: str, hdr_time: float, verbose: bool) -> str:
    s = CSRC / src
    o = OBJ / (Path(src).stem + ".o")
    if o.exists() and o.stat().st_mtime >= max(s.stat().st_mtime, hdr_time):
        return ""
    cmd = [NVCC, *ARCH, *FLAGS, "-c", str(s), "-o", str(o)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return r.stderr if verbose else ""


def build(verbose: bool = False) -> Path:
    OBJ.mkdir(exist_ok=True)
    with open(OBJ / ".lock", "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        try:
            return _build_locked(verbose)
        finally:
            fcntl.flock(lock, fcntl.LOCK_UN)


def _build_locked(verbose: bool) -> Path:
    hdr = _deps()
    jobs = min(len(SOURCES), os.cpu_count() or 4)
    with ThreadPoolExecutor(jobs) as ex:
        # the heaviest translation units first
        order = sorted(SOURCES, key=lambda x: -(CSRC / x).stat().st_size)
        for msg in ex.map(lambda f: _compile(f, hdr, verbose), order):
            if msg:
                print(msg, file=sys.stderr)
    objs = [str(OBJ / (Path(s).stem + ".o")) for s in SOURCES]
    if not LIB.exists() or LIB.stat().st_mtime < max(Path(o).stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [NVCC, *ARCH, "-shared", "-o", str(tmp), *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        tmp.replace(LIB)   # a process that has the old library loaded keeps its mapping
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
