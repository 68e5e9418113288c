"""Regenerates the golden fixtures in this folder from the reference itself.

Runs ``oracle/_ref/ref_harness`` (built by ``python oracle/build.py --ref``
from the reference headers) and stores what the reference's own functions
return:

* ``ref_sliding.jsonl`` — boards for n = 3, 4, 5 with the reference printer's
  text, the reference Manhattan value (blank included) and the result of each
  of the four moves of its successor function;
* ``ref_grid.jsonl`` — small weighted grids (sides <= 255) with the result of
  each of the eight moves of the grid successor function from sampled cells
  and the reference Manhattan value;
* ``ref_parse.jsonl`` — sliding and grid text inputs as parsed and printed by
  the reference's own readers and printers.

Only needed when the reference changes; the fixtures are committed.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import build as oracle_build  # noqa: E402

SLIDING_PARSE_CASES = {
    3: ["1,2,3,4,5,6,7,8,_ _,1,2,3,4,5,6,7,8",
        "0,1,2,3,4,5,6,7,8 1,2,3,4,5,6,7,8,0",
        "8,7,6,5,4,3,2,1,_ 1,_,2,3,4,5,6,7,8"],
    4: ["1,2,3,4,5,6,7,8,9,10,11,12,13,14,15,_ _,1,2,3,4,5,6,7,8,9,10,11,12,13,14,15",
        "15,14,13,12,11,10,9,8,7,6,5,4,3,2,1,0 0,1,2,3,4,5,6,7,8,9,10,11,12,13,14,15"],
    5: ["_,1,2,3,4,5,6,7,8,9,10,11,12,13,14,15,16,17,18,19,20,21,22,23,24 "
        "1,2,3,4,5,6,7,8,9,10,11,12,13,14,15,16,17,18,19,20,21,22,23,24,_"],
}

GRID_PARSE_CASES = [
    "5,4\n0,0\n4,3\n3\n1,1\n2,2\n1,0\n2\n3,3,7\n0,3,2\n",
    "3,3 2,2 0,0 0 0\n",
    "10,10\n9,0\n0,9\n4\n5,5 4,4 5,4 4,5\n3\n1,1,300\n2,2,9\n0,0,1\n",
]


def main() -> None:
    exe = oracle_build.build_ref_harness()
    if exe is None:
        raise SystemExit("reference tree not found; fixtures cannot be regenerated here")

    def run(args, stdin=None):
        return subprocess.run([exe, *args], input=stdin, capture_output=True, text=True,
                              check=True).stdout

    with open(os.path.join(HERE, "ref_sliding.jsonl"), "w") as f:
        f.write(run(["sliding", "3", "48", "3003"]))
        f.write(run(["sliding", "4", "48", "4004"]))
        f.write(run(["sliding", "5", "48", "5005"]))
    with open(os.path.join(HERE, "ref_grid.jsonl"), "w") as f:
        f.write(run(["grid", "14", "7007"]))
    with open(os.path.join(HERE, "ref_parse.jsonl"), "w") as f:
        for n, cases in SLIDING_PARSE_CASES.items():
            f.write(run(["parse_sliding", str(n)], "\n".join(cases) + "\n"))
        for doc in GRID_PARSE_CASES:
            out = run(["parse_grid"], doc)
            f.write(out.rstrip("\n")[:-1] + ',"input":' + _json_str(doc) + "}\n")


def _json_str(s: str) -> str:
    import json
    return json.dumps(s)


if __name__ == "__main__":
    main()
