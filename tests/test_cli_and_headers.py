"""The astar_gpu command's flag handling (no GPU needed) and a compile check
of the header-only template API against the reference's plugin types."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "cuda_a_star_gb300", "_build", "astar_gpu")


@pytest.fixture(scope="module")
def cli(gastar):
    assert os.path.exists(CLI)
    return CLI


@pytest.mark.parametrize("args,msg", [
    (["--version"], "Parameter without argument."),
    (["--version", "foo"], "Unknown version foo"),
    (["--bogus", "1"], "Unknown option --bogus"),
    (["--version", "sliding", "--heuristic", "nope"], "Unknown heuristic nope"),
])
def test_cli_rejects_bad_flags_like_the_reference(cli, args, msg):
    p = subprocess.run([cli, *args], capture_output=True, text=True)
    assert p.returncode == 255          # exit(-1), main.cu:20-24
    assert p.stdout.strip() == msg


def test_template_api_compiles():
    sys.path.insert(0, os.path.join(ROOT, "tests", "plugin"))
    import build_harness
    obj = build_harness.build(obj_only=True)
    assert os.path.getsize(obj) > 0
