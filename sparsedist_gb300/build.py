"""Build recipe of libsdgpu.so (sm_103a, nvcc, no cmake).

Each translation unit of ``csrc/`` is compiled in parallel into ``_build/``
and linked into ``sparsedist_gb300/libsdgpu.so`` (in-tree, git-ignored).
``sdg_exact.cu`` is compiled with ``-fmad=false`` so that no FP64 multiply-add
is contracted: the exact kernels must round like the reference's CPU code.

    python -m sparsedist_gb300.build          # incremental
    python -m sparsedist_gb300.build --force  # rebuild everything
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsdgpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
                      "-I", CSRC, "-I", INCLUDE]
# (source, extra flags)
UNITS = [
    ("sdg_exact.cu", ["-fmad=false"]),
    ("sdg_select.cu", []),
    ("sdg_snn.cu", []),
    ("sdg_screen.cu", []),
    ("sdg_noalloc.cu", []),
    ("sdg_dense.cu", []),
    ("sdg_dense_tc.cu", []),
    ("sdg_sparse_tc.cu", []),
    ("sdg_api.cpp", []),
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: libsdgpu.so cannot be built")


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))] + \
        [os.path.join(INCLUDE, "sdgpu.h")]


def _compile(src, extra, force):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [src] + _headers()
    if not force and os.path.exists(obj) and all(os.path.getmtime(d) <= os.path.getmtime(obj) for d in deps):
        return obj
    cmd = [nvcc(), *NVCC_COMMON, *extra, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        futs = [ex.submit(_compile, os.path.join(CSRC, s), extra, force) for s, extra in UNITS]
        objs = [f.result() for f in futs]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        cudalib = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "lib64")
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcublas",
               "-Xlinker", "-rpath", "-Xlinker", cudalib]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
        os.replace(tmp, LIB)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
