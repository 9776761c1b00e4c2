"""Build the in-tree shared library topopt_gb300/libtopopt_gb300.so.

nvcc compiles every translation unit of topopt_gb300/csrc for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, and links them into one
C-ABI shared library.  No cmake, no torch: the library depends on the CUDA
runtime alone.  Run ``python -m topopt_gb300.build`` or call ``build()``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtopopt_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["k_operator.cu", "k_vector.cu", "k_simp.cu", "k_multigrid.cu", "solver.cu", "api.cu",
           "formats.cu", "noalloc.cu", "homog.cu", "server.cu", "k_active.cu", "tune.cu",
           "k_coarse_tc.cu"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps_mtime() -> float:
    names = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    names.append(os.path.join(HERE, "..", "include", "topopt_gb300.h"))
    return max(os.path.getmtime(n) for n in names)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    newest = _deps_mtime()
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    cc = nvcc()
    # Host code computes constants the reference computes (D, weights, the OC
    # bisection); no multiply/add pair may fuse there, on any host ISA.
    flags = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                    "-Xcompiler", "-Wall", "-Xcompiler", "-ffp-contract=off",
                    "--expt-relaxed-constexpr"]

    def compile_one(src: str) -> str:
        obj = os.path.join(OBJ, src.replace(".cu", ".o"))
        cmd = [cc] + flags + ["-c", os.path.join(CSRC, src), "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{res.stdout}\n{res.stderr}")
        if verbose and (res.stdout or res.stderr):
            sys.stderr.write(res.stdout + res.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
