"""The reference's own CUDA search and its plugin headers over this engine's
template API compile for sm_103a and export their entry points (no GPU).

Skipped when the reference headers are not staged in oracle/_ref/src.  The
GPU runs of both are in test_gpu_reference_build.py.
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _exports(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if ln.strip()}


def test_reference_gpu_search_compiles():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build as oracle_build
    path = oracle_build.build_ref_gpu()
    if path is None:
        pytest.skip("reference headers not staged")
    assert {"ref_gpu_solve", "ref_gpu_error"} <= _exports(path)


def test_reference_plugins_compile_over_template_api(gastar):
    sys.path.insert(0, os.path.join(ROOT, "tests", "plugin"))
    import build_harness
    path = build_harness.build_ref_plugin()
    if path is None:
        pytest.skip("reference headers not staged")
    assert {"refplug_solve", "refplug_error"} <= _exports(path)
