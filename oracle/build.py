"""Build recipe for the CPU oracle (test infrastructure only).

* ``oracle/_build/liboracle.so`` — the C restatement (gcc, portable C11).
* ``oracle/_ref/ref_harness`` — the reference's own successor, heuristic,
  parser and printer functions compiled for the host from the reference
  headers where they lie (only when the reference tree is present; it is not
  on GPU machines, which use the committed golden fixtures instead).
* ``oracle/_ref/src/`` — the reference's headers, staged unmodified (a plain
  copy, git-ignored, never committed) so that the reference's own GA* can be
  compiled on the GPU machine, where the reference tree does not exist.
* ``oracle/_ref/libref_gpu.so`` — ``ref_gpu_harness.cu`` over the staged
  headers for sm_103a: the reference's own CUDA search, built on the machine
  that runs it.

The reference tree is the ``--reference-tree`` argument, else the
``GASTAR_REFERENCE_TREE`` environment variable, else the read-only location
the development container mounts it at (``REFERENCE_MOUNT``); only this recipe
names that location.

Usage: ``python oracle/build.py [--ref] [--stage-ref] [--ref-gpu] [--reference-tree DIR]``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
REFERENCE_MOUNT = "/root/reference"
REF_SRC = os.path.join(REF_OUT, "src")
REF_GPU_LIB = os.path.join(REF_OUT, "libref_gpu.so")
LIB = os.path.join(BUILD, "liboracle.so")
# The reference's files the search path needs (its Makefile's dependency list).
REF_FILES = ["a_star.h", "a_star_pathfinding.h", "a_star_sliding_puzzle.h", "bitonic_sort.h",
             "consts.h", "device_hashmap.h", "fancy_hashmap.h", "functional_types.h", "heaps.h",
             "helpers.h", "reduction.h", "main.cu"]


def reference_tree(tree: str | None = None) -> str:
    return tree or os.environ.get("GASTAR_REFERENCE_TREE") or REFERENCE_MOUNT


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


def build_ref_harness(force: bool = False, tree: str | None = None) -> str | None:
    """Compile oracle/ref_harness.cu against the reference headers, if present."""
    tree = reference_tree(tree)
    if not os.path.isfile(os.path.join(tree, "a_star_sliding_puzzle.h")):
        return None
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src = os.path.join(HERE, "ref_harness.cu")
    out = os.path.join(REF_OUT, "ref_harness")
    if force or _stale(out, [src]):
        os.makedirs(REF_OUT, exist_ok=True)
        cmd = [nvcc, "-std=c++17", "-O1", "-I", tree, src, "-o", out,
               "-diag-suppress", "20094"]
        subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL)
    return out


def stage_reference(tree: str | None = None) -> str | None:
    """Copy the reference's search-path files, unmodified, into oracle/_ref/src
    (git-ignored) so they travel with the working tree to the GPU machine."""
    tree = reference_tree(tree)
    if not all(os.path.isfile(os.path.join(tree, f)) for f in REF_FILES):
        return None
    os.makedirs(REF_SRC, exist_ok=True)
    for f in REF_FILES:
        dst = os.path.join(REF_SRC, f)
        src = os.path.join(tree, f)
        if not os.path.exists(dst) or os.path.getmtime(dst) < os.path.getmtime(src):
            shutil.copyfile(src, dst)
    return REF_SRC


def build_ref_gpu(force: bool = False) -> str | None:
    """Compile the reference's own GA* (staged headers + ref_gpu_harness.cu)
    for sm_103a into oracle/_ref/libref_gpu.so.  None when nothing is staged."""
    if not all(os.path.isfile(os.path.join(REF_SRC, f)) for f in REF_FILES):
        return None
    src = os.path.join(HERE, "ref_gpu_harness.cu")
    deps = [src] + [os.path.join(REF_SRC, f) for f in REF_FILES]
    if force or _stale(REF_GPU_LIB, deps):
        nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
        tmp = REF_GPU_LIB + ".tmp"
        # -std=c++14 as the reference's Makefile; sm_103a instead of its
        # compute_61, which CUDA 13 no longer accepts.
        cmd = [nvcc, "-std=c++14", "-O3", "-gencode", "arch=compute_103a,code=sm_103a",
               "-Xcompiler", "-fPIC", "-shared", "-I", REF_SRC, src, "-o", tmp,
               "-diag-suppress", "20094"]
        subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL)
        os.replace(tmp, REF_GPU_LIB)
    return REF_GPU_LIB


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--ref", action="store_true", help="host golden-vector harness")
    ap.add_argument("--stage-ref", action="store_true", help="stage the reference headers")
    ap.add_argument("--ref-gpu", action="store_true", help="the reference's GA* for sm_103a")
    ap.add_argument("--reference-tree", default=None)
    a = ap.parse_args()
    print(build_oracle(force=a.force))
    if a.ref:
        print(build_ref_harness(force=a.force, tree=a.reference_tree))
    if a.stage_ref:
        print(stage_reference(a.reference_tree))
    if a.ref_gpu:
        print(build_ref_gpu(force=a.force))
