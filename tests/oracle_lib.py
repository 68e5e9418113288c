"""ctypes binding of the CPU oracle (oracle/liboracle.so) for the test suite."""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import build as _oracle_build  # noqa: E402

ADM, REF, ZERO = 0, 1, 2
OK, NO_PATH, BUDGET, BAD_INPUT, PATH_CAP = 0, 1, 2, 3, 4


class OResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("cost", C.c_uint32), ("path_len", C.c_uint32),
                ("pad", C.c_uint32), ("expansions", C.c_uint64), ("generated", C.c_uint64),
                ("pushes", C.c_uint64), ("seconds", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(_oracle_build.build_oracle())
        u8p, u32p = C.POINTER(C.c_uint8), C.POINTER(C.c_uint32)
        _lib.oracle_sliding_successor.argtypes = [C.c_int, u8p, C.c_int, C.c_int, u8p, u32p]
        _lib.oracle_sliding_h.argtypes = [C.c_int, u8p, u8p, C.c_int]
        _lib.oracle_sliding_h.restype = C.c_uint32
        _lib.oracle_sliding_solvable.argtypes = [C.c_int, u8p, u8p]
        _lib.oracle_sliding_astar.argtypes = [C.c_int, u8p, u8p, C.c_int, C.c_int, C.c_uint64,
                                              C.POINTER(OResult), u8p, C.c_uint32]
        _lib.oracle_sliding_validate.argtypes = [C.c_int, u8p, u8p, u8p, C.c_uint32, C.c_int, u32p]
        _lib.oracle_bfs8.argtypes = [u8p, u8p]
        _lib.oracle_perm_rank9.argtypes = [u8p]
        _lib.oracle_perm_rank9.restype = C.c_uint32
        _lib.oracle_grid_successor.argtypes = [C.c_uint32, C.c_uint32, u8p, C.c_uint32, C.c_uint32,
                                               C.c_int, u32p, u32p, u32p]
        _lib.oracle_grid_h.argtypes = [C.c_uint32] * 5 + [C.c_int]
        _lib.oracle_grid_h.restype = C.c_uint32
        _lib.oracle_grid_astar.argtypes = [C.c_uint32, C.c_uint32, u8p, C.c_uint32, C.c_uint32,
                                           C.c_uint32, C.c_uint32, C.c_int, C.c_uint64,
                                           C.POINTER(OResult), u32p, C.c_uint32]
        _lib.oracle_grid_validate.argtypes = [C.c_uint32, C.c_uint32, u8p, C.c_uint32, C.c_uint32,
                                              C.c_uint32, C.c_uint32, u32p, C.c_uint32, u32p]
        _lib.oracle_sliding_batch.argtypes = [C.c_int, C.c_uint32, u8p, u8p, C.c_int, C.c_int,
                                              C.POINTER(OResult)]
        _lib.oracle_grid_batch.argtypes = [C.c_uint32, u8p, C.POINTER(C.c_uint64), u32p, u32p,
                                           C.c_int, C.c_int, C.POINTER(OResult)]
    return _lib


def _u8(a):
    a = np.ascontiguousarray(a, dtype=np.uint8)
    return a, a.ctypes.data_as(C.POINTER(C.c_uint8))


def _u32(a):
    a = np.ascontiguousarray(a, dtype=np.uint32)
    return a, a.ctypes.data_as(C.POINTER(C.c_uint32))


def sliding_successor(n, board, move, ref_moves=0):
    b, bp = _u8(board)
    out = np.zeros(n * n, np.uint8)
    cost = C.c_uint32()
    ex = lib().oracle_sliding_successor(n, bp, move, ref_moves, out.ctypes.data_as(C.POINTER(C.c_uint8)),
                                        C.byref(cost))
    return bool(ex), cost.value, out


def sliding_h(n, board, goal, heuristic):
    b, bp = _u8(board)
    g, gp = _u8(goal)
    return lib().oracle_sliding_h(n, bp, gp, heuristic)


def sliding_solvable(n, start, goal):
    s, sp = _u8(start)
    g, gp = _u8(goal)
    return bool(lib().oracle_sliding_solvable(n, sp, gp))


def sliding_astar(n, start, goal, heuristic=ADM, ref_moves=0, max_exp=0, path=True):
    s, sp = _u8(start)
    g, gp = _u8(goal)
    r = OResult()
    cap = 4096 if path else 0
    buf = np.zeros((max(cap, 1), n * n), np.uint8)
    lib().oracle_sliding_astar(n, sp, gp, heuristic, ref_moves, max_exp, C.byref(r),
                               buf.ctypes.data_as(C.POINTER(C.c_uint8)) if path else None, cap)
    p = buf[:r.path_len].copy() if (path and r.status == OK) else None
    return r, p


def sliding_validate(n, start, goal, path, ref_moves=0):
    s, sp = _u8(start)
    g, gp = _u8(goal)
    p, pp = _u8(np.asarray(path).reshape(-1))
    cost = C.c_uint32()
    ok = lib().oracle_sliding_validate(n, sp, gp, pp, len(path), ref_moves, C.byref(cost))
    return bool(ok), cost.value


def bfs8(goal):
    g, gp = _u8(goal)
    dist = np.zeros(362880, np.uint8)
    cnt = lib().oracle_bfs8(gp, dist.ctypes.data_as(C.POINTER(C.c_uint8)))
    return cnt, dist


def perm_rank9(board):
    b, bp = _u8(board)
    return lib().oracle_perm_rank9(bp)


def grid_successor(weights, x, y, move):
    w8, wp = _u8(weights)
    h, w = w8.shape
    nx, ny, c = C.c_uint32(), C.c_uint32(), C.c_uint32()
    ex = lib().oracle_grid_successor(w, h, wp, x, y, move, C.byref(nx), C.byref(ny), C.byref(c))
    return bool(ex), nx.value, ny.value, c.value


def grid_h(x, y, tx, ty, minw, heuristic):
    return lib().oracle_grid_h(x, y, tx, ty, minw, heuristic)


def grid_astar(weights, start, goal, heuristic=ADM, max_exp=0, path=True):
    w8, wp = _u8(weights)
    h, w = w8.shape
    r = OResult()
    cap = w * h if path else 0
    buf = np.zeros(max(cap, 1), np.uint32)
    lib().oracle_grid_astar(w, h, wp, start[0], start[1], goal[0], goal[1], heuristic, max_exp,
                            C.byref(r), buf.ctypes.data_as(C.POINTER(C.c_uint32)) if path else None, cap)
    p = buf[:r.path_len].copy() if (path and r.status == OK) else None
    return r, p


def grid_validate(weights, start, goal, path):
    w8, wp = _u8(weights)
    h, w = w8.shape
    p, pp = _u32(np.asarray(path))
    cost = C.c_uint32()
    ok = lib().oracle_grid_validate(w, h, wp, start[0], start[1], goal[0], goal[1], pp, len(p),
                                    C.byref(cost))
    return bool(ok), cost.value


def sliding_batch(n, starts, goals, heuristic=ADM, threads=0):
    s, sp = _u8(np.asarray(starts).reshape(-1))
    g, gp = _u8(np.asarray(goals).reshape(-1))
    count = len(s) // (n * n)
    res = (OResult * count)()
    used = lib().oracle_sliding_batch(n, count, sp, gp, heuristic, threads, res)
    return used, list(res)


def grid_batch(grids, heuristic=ADM, threads=0):
    """grids: list of (weights, start, goal)."""
    flat, offs, dims, ends = [], [], [], []
    off = 0
    for wts, st, gl in grids:
        wts = np.ascontiguousarray(wts, np.uint8)
        flat.append(wts.reshape(-1))
        offs.append(off)
        off += wts.size
        dims += [wts.shape[1], wts.shape[0]]
        ends += [st[0], st[1], gl[0], gl[1]]
    w, wp = _u8(np.concatenate(flat))
    o = np.asarray(offs, np.uint64)
    d, dp = _u32(dims)
    e, ep = _u32(ends)
    res = (OResult * len(grids))()
    used = lib().oracle_grid_batch(len(grids), wp, o.ctypes.data_as(C.POINTER(C.c_uint64)), dp, ep,
                                   heuristic, threads, res)
    return used, list(res)
