"""libgastar.so loads, exports every declared symbol, and its host-only
functions (parsers, printers, generators) behave -- no GPU call is made."""
import json
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def _declared():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(gastar_[a-z0-9_]+)\s*\(", src))
    return names


def test_exports_every_declared_symbol(gastar):
    from cuda_a_star_gb300 import _lib
    lib = gastar.lib()
    declared = _declared()
    assert declared, "no declarations found"
    for name in sorted(declared):
        assert hasattr(lib, name), name
    assert declared == set(_lib.EXPORTS)


def test_no_cpu_fallback_when_library_missing(tmp_path):
    from cuda_a_star_gb300 import _lib
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        saved = _lib._lib
        _lib._lib = None
        try:
            _lib.load(str(tmp_path / "missing.so"))
        finally:
            _lib._lib = saved


def _golden_parse():
    with open(os.path.join(GOLDEN, "ref_parse.jsonl")) as f:
        return [json.loads(l) for l in f if l.strip()]


@pytest.mark.parametrize("rec", [r for r in _golden_parse() if r["kind"] == "sliding_parse"],
                         ids=lambda r: r["input"][0])
def test_sliding_parser_matches_reference(gastar, rec):
    n = rec["n"]
    s, g = gastar.parse_sliding(" ".join(rec["input"]), n)
    assert s.tolist() == rec["start"] and g.tolist() == rec["goal"]
    assert gastar.format_sliding(s) == rec["printed"][0]
    assert gastar.format_sliding(g) == rec["printed"][1]


@pytest.mark.parametrize("rec", [r for r in _golden_parse() if r["kind"] == "grid_parse"],
                         ids=lambda r: r["board"])
def test_grid_parser_matches_reference(gastar, rec):
    wts, st, gl = gastar.parse_grid(rec["input"])
    w, h = map(int, rec["board"].split(","))
    assert wts.shape == (h, w)
    assert st == tuple(map(int, rec["start"].split(",")))
    assert gl == tuple(map(int, rec["target"].split(",")))
    expect = np.ones((h, w), np.uint8)
    for x, y, c in rec["costs"]:
        expect[y, x] = c
    for x, y in rec["obstacles"]:
        expect[y, x] = 0
    assert (wts == expect).all()


def test_parser_errors(gastar):
    with pytest.raises(gastar.GastarError):
        gastar.parse_sliding("1,2,3 4,5,6", 3)
    with pytest.raises(gastar.GastarError):
        gastar.parse_sliding("1,1,2,3,4,5,6,7,8 0,1,2,3,4,5,6,7,8", 3)
    with pytest.raises(gastar.GastarError):
        gastar.parse_grid("3,3 0,0 5,5 0 0")
    with pytest.raises(gastar.GastarError):
        gastar.parse_grid("3,3 0,0 1,1 0 1 1,1,0")


def test_generators_deterministic_and_well_formed(gastar, oracle):
    s1, g1 = gastar.gen_sliding(4, 42, 40, 80)
    s2, g2 = gastar.gen_sliding(4, 42, 40, 80)
    assert (s1 == s2).all() and (g1 == g2).all()
    assert g1.tolist() == list(range(16))
    assert sorted(s1.tolist()) == list(range(16))
    assert oracle.sliding_solvable(4, s1, g1)
    w = gastar.gen_grid(64, 48, 9, 0.3)
    assert w.shape == (48, 64) and w.max() <= 9
    assert 0.2 < (w == 0).mean() < 0.4
    r, p = oracle.grid_astar(w, (0, 0), (63, 47))
    assert r.status == oracle.OK   # the corridor guarantees a path
    assert (gastar.gen_grid(64, 48, 9, 0.3) == w).all()
