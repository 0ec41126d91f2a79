"""Builds libaran_gpu.so in-tree with nvcc for sm_103a.

Each translation unit compiles in its own process (in parallel), then one
link step writes ``aran_gb300/libaran_gpu.so``.  Objects go to ``_build/``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(ROOT, "_build", "aran_gpu")
LIB = os.path.join(HERE, "libaran_gpu.so")
SOURCES = ["tables.cu", "tree.cu", "passes.cu", "p2p.cu", "m2l.cu", "m2l_lanes.cu", "m2l_tc.cu", "m2m_lanes.cu", "kkylin.cu",
           "noalloc.cu", "server.cu", "solver.cu", "compat.cu", "solver2d.cu", "compat2d.cu",
           "semifar.cu", "series3d.cu", "tune.cu", "profiledb.cpp"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
         "-I/usr/local/cuda/include/cccl", "-I" + os.path.join(ROOT, "include"),
         "--expt-relaxed-constexpr"]


def _deps() -> list[str]:
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".cpp"))]
    for sub in ("", "aran", "vsg"):
        d = os.path.join(ROOT, "include", sub)
        out += [os.path.join(d, f) for f in os.listdir(d) if f.endswith(".h")]
    return out


def _compile(src: str) -> str:
    obj = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    cmd = [NVCC] + ARCH + FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False) -> str:
    """Compile (if sources changed) and return the path of libaran_gpu.so."""
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in _deps()):
            return LIB
    os.makedirs(OBJ, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
