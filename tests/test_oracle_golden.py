"""The oracle against vectors produced by the reference's own functions.

tests/golden/*.jsonl come from tests/golden/make_golden.py, which compiles the
reference's successor, heuristic, parser and printer functions for the host
(oracle/ref_harness.cu) and records their outputs.
"""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return [json.loads(line) for line in f if line.strip()]


SLIDING = _load("ref_sliding.jsonl")
GRID = _load("ref_grid.jsonl")
PARSE = _load("ref_parse.jsonl")


def test_fixture_sizes():
    assert {r["n"] for r in SLIDING} == {3, 4, 5}
    assert len(SLIDING) == 144 and len(GRID) == 14


@pytest.mark.parametrize("rec", SLIDING, ids=lambda r: f"n{r['n']}-{r['printed']}")
def test_sliding_successor_ref_moves_bit_exact(oracle, rec):
    """ref_moves reproduces the reference's successor function exactly."""
    n, board = rec["n"], np.array(rec["board"], np.uint8)
    for m, mv in enumerate(rec["moves"]):
        ex, cost, nxt = oracle.sliding_successor(n, board, m, ref_moves=1)
        assert ex == bool(mv["exists"]), (m, mv)
        assert cost == mv["cost"]
        if ex:
            assert nxt.tolist() == mv["next"]


@pytest.mark.parametrize("rec", SLIDING, ids=lambda r: f"n{r['n']}-{r['printed']}")
def test_sliding_successor_standard_moves(oracle, rec):
    """Standard moves agree with the reference on moves 0 and 2 (the only ones
    the reference's arithmetic lets through) and mirror them for 1 and 3."""
    n, board = rec["n"], np.array(rec["board"], np.uint8)
    blank = int(np.flatnonzero(board == 0)[0])
    assert [blank // n, blank % n] == rec["blank"]
    for m, mv in enumerate(rec["moves"]):
        ex, cost, nxt = oracle.sliding_successor(n, board, m, ref_moves=0)
        if m in (0, 2):
            assert ex == bool(mv["exists"])
            if ex:
                assert nxt.tolist() == mv["next"]
        else:
            assert mv["exists"] == 0  # the reference never produces moves 1 and 3
            r, c = blank // n, blank % n
            expect = (r > 0) if m == 1 else (c > 0)
            assert ex == expect
            if ex:  # the inverse of the move back must restore the board
                back_ok, _, back = oracle.sliding_successor(n, nxt, m ^ 1, ref_moves=0)
                assert back_ok and back.tolist() == board.tolist()


@pytest.mark.parametrize("rec", SLIDING, ids=lambda r: f"n{r['n']}-{r['printed']}")
def test_sliding_heuristic_reference_formula(oracle, rec):
    n = rec["n"]
    b, g = np.array(rec["board"], np.uint8), np.array(rec["goal"], np.uint8)
    assert oracle.sliding_h(n, b, g, oracle.REF) == rec["h_ref"]
    # admissible variant = reference value minus the blank's own distance
    gb = int(np.flatnonzero(g == 0)[0])
    bb = int(np.flatnonzero(b == 0)[0])
    blank_d = abs(gb // n - bb // n) + abs(gb % n - bb % n)
    assert oracle.sliding_h(n, b, g, oracle.ADM) == rec["h_ref"] - blank_d


@pytest.mark.parametrize("rec", GRID, ids=lambda r: f"{r['w']}x{r['h']}")
def test_grid_successor_bit_exact(oracle, rec):
    w, h = rec["w"], rec["h"]
    wts = np.array(rec["weights"], np.uint8).reshape(h, w)
    tx, ty = rec["target"]
    for cell in rec["cells"]:
        assert oracle.grid_h(cell["x"], cell["y"], tx, ty, 1, oracle.REF) == cell["h_ref"]
        for m, mv in enumerate(cell["moves"]):
            ex, nx, ny, cost = oracle.grid_successor(wts, cell["x"], cell["y"], m)
            assert ex == bool(mv["exists"]), (cell, m)
            if ex:
                assert (nx, ny, cost) == (mv["x"], mv["y"], mv["cost"])


def test_parse_records_present():
    kinds = {r["kind"] for r in PARSE}
    assert kinds == {"sliding_parse", "grid_parse"}
