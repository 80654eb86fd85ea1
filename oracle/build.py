"""Build recipe for the CPU oracle (test infrastructure only).

* ``build_oracle()`` compiles the C restatement ``oracle/sdg_oracle.c`` into
  ``oracle/_build/libsdgoracle.so`` (gcc, OpenMP, ``-ffp-contract=off`` so that
  no multiply-add is fused on any host, x86-64 or aarch64).
* ``build_ref()`` compiles the reference's own, unmodified hot-path sources
  (``src/sparseDist.cpp``, ``src/topK.cpp``, ``src/topKRows.cpp``,
  ``src/snn.cpp`` of gambalab/sparseDist) where they lie, against the
  project-written API shim in ``oracle/shim/``, into ``oracle/_ref/libsdref.so``.
  It needs the reference checkout: ``$SDG_REFERENCE_ROOT`` if set, else a
  ``reference`` directory beside this repository's root; where neither holds
  the sources it does nothing.

Run ``python oracle/build.py`` or call the functions.  Nothing under
``oracle/`` is part of the product.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "libsdgoracle.so")
REF_SO = os.path.join(REF_DIR, "libsdref.so")
REF_SOURCES = ("sparseDist.cpp", "topK.cpp", "topKRows.cpp", "snn.cpp")
# the reference checkout when SDG_REFERENCE_ROOT is unset: a sibling of the
# repository root
SIBLING_REF_ROOT = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")

COMMON = ["-O2", "-fopenmp", "-ffp-contract=off", "-fPIC"]


def _run(cmd):
    subprocess.run(cmd, check=True)


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_oracle(force: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    src = os.path.join(HERE, "sdg_oracle.c")
    deps = [src, os.path.join(HERE, "sdg_oracle.h")]
    if force or _stale(ORACLE_SO, deps):
        _run(["gcc", *COMMON, "-shared", "-o", ORACLE_SO, src, "-lm"])
    return ORACLE_SO


def build_ref(ref_root: str | None = None, force: bool = False) -> str | None:
    ref_root = ref_root or os.environ.get("SDG_REFERENCE_ROOT") or SIBLING_REF_ROOT
    srcs = [os.path.join(ref_root, "src", s) for s in REF_SOURCES]
    if not all(os.path.exists(s) for s in srcs):
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    shim = os.path.join(HERE, "shim")
    driver = os.path.join(HERE, "ref_driver.cpp")
    orc_c = os.path.join(HERE, "sdg_oracle.c")
    deps = srcs + [driver, orc_c, os.path.join(shim, "sdg_shim.hpp")]
    if not (force or _stale(REF_SO, deps)):
        return REF_SO
    orc_o = os.path.join(REF_DIR, "sdg_oracle.o")
    _run(["gcc", *COMMON, "-c", "-o", orc_o, orc_c])
    _run(["g++", *COMMON, "-std=c++17", "-DARMA_64BIT_WORD=1", "-w", "-I", shim,
          "-shared", "-o", REF_SO, *srcs, driver, orc_o, "-lm"])
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
