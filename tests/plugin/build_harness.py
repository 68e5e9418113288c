"""Builds tests/plugin/plugin_harness.cu into tests/plugin/_build/ (test infrastructure)."""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def build(obj_only: bool = False) -> str:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    src = os.path.join(HERE, "plugin_harness.cu")
    lib_dir = os.path.join(ROOT, "cuda_a_star_gb300", "_build")
    common = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
              "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"), "--expt-relaxed-constexpr"]
    if obj_only:
        out = os.path.join(out_dir, "plugin_harness.o")
        subprocess.run(common + ["-c", src, "-o", out], check=True)
        return out
    out = os.path.join(out_dir, "libplugin_harness.so")
    if os.path.exists(out) and os.path.getmtime(out) > max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(lib_dir, "libgastar.so"))):
        return out
    subprocess.run(common + ["-shared", src, "-o", out, "-L", lib_dir, "-lgastar",
                             "-Xlinker", "-rpath=" + lib_dir], check=True)
    return out


def build_ref_plugin() -> str | None:
    """tests/plugin/ref_plugin_harness.cu: the reference's own plugin headers,
    staged unmodified in oracle/_ref/src, over include/gastar/a_star.cuh.
    None when the reference headers are not staged."""
    ref_src = os.path.join(ROOT, "oracle", "_ref", "src")
    if not os.path.isfile(os.path.join(ref_src, "a_star_pathfinding.h")):
        return None
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    src = os.path.join(HERE, "ref_plugin_harness.cu")
    out = os.path.join(out_dir, "libref_plugin_harness.so")
    deps = [src, os.path.join(ref_src, "a_star_pathfinding.h"),
            os.path.join(ref_src, "a_star_sliding_puzzle.h"),
            os.path.join(ROOT, "include", "gastar", "a_star.cuh")]
    if os.path.exists(out) and os.path.getmtime(out) > max(os.path.getmtime(d) for d in deps):
        return out
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
                    "-Xcompiler", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"),
                    "-I", ref_src, "--expt-relaxed-constexpr", "-diag-suppress", "20094",
                    src, "-o", out], check=True)
    return out
