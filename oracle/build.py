"""Build recipe for the CPU oracle (test infrastructure only).

* ``oracle/_build/liboracle.so`` — the C restatement (gcc, portable C11).
* ``oracle/_ref/ref_harness`` — the reference's own successor, heuristic,
  parser and printer functions compiled for the host from the reference
  headers where they lie (only when the reference tree is present; it is not
  on GPU machines, which use the committed golden fixtures instead).

Usage: ``python oracle/build.py [--ref]``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
REFERENCE_TREE = os.environ.get("GASTAR_REFERENCE_TREE", "/root/reference")
LIB = os.path.join(BUILD, "liboracle.so")


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force: bool = False) -> str:
    srcs = [os.path.join(HERE, "oracle.c"), os.path.join(HERE, "oracle.h")]
    if force or _stale(LIB, srcs):
        os.makedirs(BUILD, exist_ok=True)
        tmp = LIB + ".tmp"
        cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-pthread",
               srcs[0], "-o", tmp]
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


def build_ref_harness(force: bool = False) -> str | None:
    """Compile oracle/ref_harness.cu against the reference headers, if present."""
    if not os.path.isfile(os.path.join(REFERENCE_TREE, "a_star_sliding_puzzle.h")):
        return None
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src = os.path.join(HERE, "ref_harness.cu")
    out = os.path.join(REF_OUT, "ref_harness")
    if force or _stale(out, [src]):
        os.makedirs(REF_OUT, exist_ok=True)
        cmd = [nvcc, "-std=c++17", "-O1", "-I", REFERENCE_TREE, src, "-o", out,
               "-diag-suppress", "20094"]
        subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL)
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    if "--ref" in sys.argv:
        print(build_ref_harness(force="--force" in sys.argv))
