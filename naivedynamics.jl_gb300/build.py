"""Build libnaivegpu.so (sm_103a) in-tree.

    python naivedynamics.jl_gb300/build.py [--verbose-ptxas]

Each .cu translation unit compiles in parallel with nvcc for sm_103a only and
the objects are linked into naivedynamics.jl_gb300/lib/libnaivegpu.so.  No
fast-math: the neighbour-search kernels rely on IEEE single precision with the
reference's operation order (explicit __f*_rn intrinsics where it matters).
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIB_DIR, "libnaivegpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["nd_bvh.cu", "nd_md.cu", "nd_adjoint.cu", "nd_capi.cu", "nd_noalloc.cu", "nd_compat.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, verbose_ptxas: bool) -> tuple[str, str]:
    out = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    # host code: no FMA contraction, so the host-side generators give the same
    # bits on x86 and on Arm hosts (device code is unaffected)
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-Wall", "-Xcompiler", "-ffp-contract=off", "-c",
           os.path.join(CSRC, src), "-o", out]
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return out, r.stderr


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "naivegpu.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    if not force and not verbose_ptxas and not _stale():
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose_ptxas), SOURCES))
    if verbose_ptxas:
        for (_, log) in results:
            sys.stderr.write(log)
    objs = [o for (o, _) in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose-ptxas", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose_ptxas=a.verbose_ptxas))
