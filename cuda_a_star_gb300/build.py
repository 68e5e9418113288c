"""Builds libgastar.so (the GA* engine) in-tree with nvcc for sm_103a.

Translation units compile in parallel, then link into
``cuda_a_star_gb300/_build/libgastar.so``.  Rebuilds only when a source or
header is newer than the library.  ``python -m cuda_a_star_gb300.build
[--force] [--verbose]``; ``--ptxas`` prints register/shared-memory usage.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgastar.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgastar")
    return cand


def sources() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def headers() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
                  glob.glob(os.path.join(ROOT, "include", "*.h")) +
                  glob.glob(os.path.join(ROOT, "include", "gastar", "*.cuh")))


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas: bool = False) -> str:
    srcs = sources()
    if not force and not _stale(LIB, srcs + headers() + [__file__]):
        if _stale(CLI, [os.path.join(HERE, "cli", "astar_gpu.cpp"), LIB]):
            build_cli(verbose)
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    common = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I", CSRC,
              "-I", os.path.join(ROOT, "include")]
    procs = []
    objs = []
    for s in srcs:
        obj = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(obj)
        cmd = [nvcc, *ARCH, *common, "-c", s, "-o", obj]
        if s.endswith(".cu"):
            cmd += ["--expt-relaxed-constexpr"]
            if ptxas:
                cmd += ["-Xptxas", "-v"]
        if verbose:
            print(" ".join(cmd))
        procs.append((s, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                                          text=True)))
    failed = []
    for s, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((s, out))
        elif (verbose or ptxas) and out.strip():
            print(out)
    if failed:
        msg = "\n".join(f"--- {s}\n{o}" for s, o in failed)
        raise RuntimeError(f"nvcc failed:\n{msg}")
    tmp = LIB + ".tmp"
    link = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    if verbose:
        print(" ".join(link))
    subprocess.run(link, check=True)
    os.replace(tmp, LIB)
    build_cli(verbose)
    return LIB


CLI = os.path.join(BUILD, "astar_gpu")


def build_cli(verbose: bool = False) -> str:
    """The astar_gpu command (host C++ over the C ABI), next to the library."""
    src = os.path.join(HERE, "cli", "astar_gpu.cpp")
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), src, "-o", CLI,
           "-L", BUILD, "-lgastar", "-Wl,-rpath,$ORIGIN"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return CLI


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv,
                ptxas="--ptxas" in sys.argv))
