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


def test_python_structs_match_the_c_header(tmp_path):
    """The ctypes mirrors of the C ABI's structs have the header's sizes and
    field offsets (gcc on include/gastar.h; no GPU)."""
    import ctypes as C
    sys.path.insert(0, ROOT)
    from cuda_a_star_gb300 import _lib
    structs = {"gastar_config": _lib.Config, "gastar_result": _lib.Result,
               "gastar_batch_config": _lib.BatchConfig}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gastar.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        cname, field, val = line.split()
        got[(cname, field)] = int(val)
    for cname, py in structs.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
