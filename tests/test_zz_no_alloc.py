"""The allocation-free 8-puzzle entry point against gastar_solve_sliding.

gastar_solve_sliding_noalloc serves callers that cannot call cudaMalloc (device
memory reserved by another pool, or no device-wide synchronisation allowed):
it runs on a fixed scratch array inside the library.  Called through the C ABI
twice in a row per instance (the second call finds the previous call's data
in the shared array), its costs and statuses must equal the existing entry
point's exactly, and its paths must be valid move by move.  Covered: the
admissible and zero heuristics, the reference's two-move successor rule
(checked against the oracle), no path buffer, a path buffer that is too small,
a caller stream, and device memory that stays the same over repeated calls.
This file is collected last so that a stop-at-first-failure run has run
everything else.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOAL = np.arange(9, dtype=np.uint8)


def _noalloc(gastar, start, goal, n=3, path=True, path_cap=64, **cfg_kw):
    lib = gastar.lib()
    s = np.ascontiguousarray(start, np.uint8)
    g = np.ascontiguousarray(goal, np.uint8)
    cfg = gastar.make_config(**cfg_kw)
    res = gastar.Result()
    buf = np.zeros((max(path_cap, 1), n * n), np.uint8)
    u8 = C.POINTER(C.c_uint8)
    rc = lib.gastar_solve_sliding_noalloc(n, s.ctypes.data_as(u8), g.ctypes.data_as(u8),
                                          C.byref(cfg), buf.ctypes.data_as(u8) if path else None,
                                          path_cap if path else 0, C.byref(res))
    ok = path and res.status == gastar.OK
    return rc, res, (buf[:res.path_len] if ok else None)


def _boards(gastar, count=10, seed=2024):
    rng = np.random.default_rng(seed)
    boards = [rng.permutation(9).astype(np.uint8) for _ in range(count)]
    boards += [gastar.gen_sliding(3, 77 + i, 60, 60)[0] for i in range(4)]
    boards.append(GOAL.copy())
    return boards


@pytest.mark.parametrize("heuristic", [0, 2], ids=["admissible", "zero"])
def test_no_alloc_matches_existing_entry_point(engine, oracle, gastar, heuristic):
    for s in _boards(gastar):
        ref = engine.solve_sliding(s, GOAL, 3, heuristic=heuristic)
        for _ in range(2):  # two calls in a row share the static scratch
            rc, r, path = _noalloc(gastar, s, GOAL, heuristic=heuristic)
            assert rc == 0
            assert (r.status, r.cost) == (ref.status, ref.cost)
            if r.status == gastar.OK:
                assert oracle.sliding_validate(3, s, GOAL, path) == (True, r.cost)
                assert len(path) == r.cost + 1


def _two_move_walk(start, steps, rng):
    """A goal reachable from `start` with the reference's two live moves
    (blank row+1, blank col+1), a_star_sliding_puzzle.h:106-111."""
    b = start.copy().reshape(3, 3)
    for _ in range(steps):
        r, c = map(int, np.argwhere(b == 0)[0])
        opts = [(r + 1, c)] if r < 2 else []
        opts += [(r, c + 1)] if c < 2 else []
        if not opts:
            break
        nr, nc = opts[int(rng.integers(len(opts)))]
        b[r, c], b[nr, nc] = b[nr, nc], 0
    return b.reshape(-1)


def test_no_alloc_reference_moves_against_oracle(engine, oracle, gastar):
    rng = np.random.default_rng(7)
    for k in range(8):
        start = rng.permutation(9).astype(np.uint8)
        if k % 2 == 0:  # blank in the top-left corner: the longest two-move walks
            z = int(np.argwhere(start == 0)[0][0])
            start[z], start[0] = start[0], 0
        goal = _two_move_walk(start, int(rng.integers(0, 5)), rng)
        ref, _ = oracle.sliding_astar(3, start, goal, heuristic=0, ref_moves=1, path=False)
        plain = engine.solve_sliding(start, goal, 3, moves=1)
        for _ in range(2):
            rc, r, path = _noalloc(gastar, start, goal, moves=1)
            assert rc == 0
            assert (r.status, r.cost) == (ref.status, ref.cost) == (plain.status, plain.cost)
            assert oracle.sliding_validate(3, start, goal, path, ref_moves=1) == (True, r.cost)
    # a goal the two moves cannot reach: the search space runs dry
    start = np.array([1, 2, 3, 4, 0, 5, 6, 7, 8], np.uint8)
    goal = np.array([0, 1, 2, 3, 4, 5, 6, 7, 8], np.uint8)
    rc, r, _ = _noalloc(gastar, start, goal, moves=1)
    assert rc == 0 and r.status == gastar.NO_PATH
    assert engine.solve_sliding(start, goal, 3, moves=1).status == gastar.NO_PATH


def test_no_alloc_without_path_and_with_a_short_buffer(engine, gastar):
    s = gastar.gen_sliding(3, 4242, 60, 60)[0]
    ref = engine.solve_sliding(s, GOAL, 3)
    assert ref.status == gastar.OK and ref.cost > 4
    rc, r, path = _noalloc(gastar, s, GOAL, path=False)
    assert rc == 0 and (r.status, r.cost) == (gastar.OK, ref.cost) and path is None
    # too short a buffer: the cost stands, path_len says what is needed
    short = engine.solve_sliding(s, GOAL, 3, path_cap=3)
    rc, r, _ = _noalloc(gastar, s, GOAL, path_cap=3)
    assert rc == 0
    assert (r.status, r.cost, r.path_len) == (short.status, ref.cost, ref.cost + 1)
    assert r.status == gastar.STATUS.index("PATH_CAP")


def test_no_alloc_on_a_caller_stream_allocates_nothing(engine, oracle, gastar):
    torch = pytest.importorskip("torch")
    stream = torch.cuda.Stream()
    boards = _boards(gastar, count=6, seed=99)
    # the first call may load the library's device module (and its array)
    _noalloc(gastar, boards[0], GOAL, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for s in boards * 2:
        rc, r, path = _noalloc(gastar, s, GOAL, stream=stream.cuda_stream)
        assert rc == 0
        ref, _ = oracle.sliding_astar(3, s, GOAL, path=False)
        assert (r.status, r.cost) == (ref.status, ref.cost)
        if r.status == gastar.OK:
            assert oracle.sliding_validate(3, s, GOAL, path) == (True, r.cost)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_no_alloc_rejects_boards_above_its_limit(gastar):
    s, g = gastar.gen_sliding(4, 5, 10, 10)
    rc, r, _ = _noalloc(gastar, s, g, n=4)
    assert rc == gastar.STATUS.index("BAD_INPUT")
    assert b"only 3x3" in gastar.lib().gastar_last_error()
