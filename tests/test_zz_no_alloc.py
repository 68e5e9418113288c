"""The allocation-free 8-puzzle entry point against gastar_solve_sliding.

gastar_solve_sliding_noalloc serves callers that cannot call cudaMalloc (device
memory reserved by another pool, or no device-wide synchronisation allowed):
it runs on a fixed scratch array inside the library.  Called through the C ABI
twice in a row per instance (the second call finds the previous call's data
in the shared array), its costs and statuses must equal the existing entry
point's exactly, and its paths must be valid move by move.  This file is
collected last so that a stop-at-first-failure run has run everything else.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(gastar, start, goal, n=3):
    lib = gastar.lib()
    s = np.ascontiguousarray(start, np.uint8)
    g = np.ascontiguousarray(goal, np.uint8)
    cfg = gastar.make_config()
    res = gastar.Result()
    path = np.zeros((64, n * n), np.uint8)
    u8 = C.POINTER(C.c_uint8)
    rc = lib.gastar_solve_sliding_noalloc(n, s.ctypes.data_as(u8), g.ctypes.data_as(u8),
                                          C.byref(cfg), path.ctypes.data_as(u8), 64, C.byref(res))
    return rc, res, path[:res.path_len]


def test_no_alloc_matches_existing_entry_point(engine, oracle, gastar):
    goal = np.arange(9, dtype=np.uint8)
    rng = np.random.default_rng(2024)
    boards = [rng.permutation(9).astype(np.uint8) for _ in range(10)]
    boards += [gastar.gen_sliding(3, 77 + i, 60, 60)[0] for i in range(4)]
    boards.append(goal.copy())
    for s in boards:
        ref = engine.solve_sliding(s, goal, 3)
        for _ in range(2):  # two calls in a row share the static scratch
            rc, r, path = _noalloc(gastar, s, goal)
            assert rc == 0
            assert (r.status, r.cost) == (ref.status, ref.cost)
            if r.status == gastar.OK:
                assert oracle.sliding_validate(3, s, goal, path) == (True, r.cost)
                assert len(path) == r.cost + 1


def test_no_alloc_rejects_boards_above_its_limit(gastar):
    s, g = gastar.gen_sliding(4, 5, 10, 10)
    rc, r, _ = _noalloc(gastar, s, g, n=4)
    assert rc == gastar.STATUS.index("BAD_INPUT")
    assert b"only 3x3" in gastar.lib().gastar_last_error()
