"""A model of the grid path walker (walk_grid_warp in search.cuh), run on the
CPU: window placement from path_win_origin, the window loads (bounded by the
grid), and lane 0's walk inside the window, with every shared-memory index
asserted in range.  On random parent chains -- grids narrower and shorter
than the window, starts and goals on edges and corners, chains that move
away from the start -- it must return the chain goal-first, and 0 for a
damaged table (a move off the grid, a missing move, a cycle past the
limit).  The window constants come from search.cuh."""
import os
import random
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EMPTY = (1 << 64) - 1
DX = [1, -1, 0, 0, 1, 1, -1, -1]  # GridDom::dx
DY = [0, 0, 1, -1, 1, -1, 1, -1]  # GridDom::dy


SRC = open(os.path.join(ROOT, "cuda_a_star_gb300", "csrc", "search.cuh")).read()


def _constants():
    m = re.search(r"constexpr int kPathWin = (\d+), kPathMargin = (\d+)", SRC)
    return int(m.group(1)), int(m.group(2))


def _pack(name):
    expr = re.search(r"constexpr uint32_t %s = ([^;]+);" % name, SRC).group(1)
    return eval(re.sub(r"(\d+)u", r"\1", expr))


WIN, MARGIN = _constants()
DXP, DYP = _pack("kGridDxPack"), _pack("kGridDyPack")


def origin(c, s, n):
    o = c - (WIN - 1 - MARGIN) if s < c else c - MARGIN if s > c else c - WIN // 2
    if o > n - WIN:
        o = n - WIN
    return max(o, 0)


def walk(table, W, H, start, goal, limit, cap=None):
    sx, sy = start % W, start // W
    cx, cy = goal % W, goal // W
    out, n, loads = [], 0, 0
    while True:
        x0, y0 = origin(cx, sx, W), origin(cy, sy, H)
        assert x0 <= cx < x0 + WIN and y0 <= cy < y0 + WIN
        win = [[table[(y0 + r) * W + x0 + j] if x0 + j < W and y0 + r < H else EMPTY
                for j in range(WIN)] for r in range(WIN)]
        loads += 1
        while True:
            assert 0 <= cy - y0 < WIN and 0 <= cx - x0 < WIN  # shared-memory index
            if cap is None or n < cap:
                out.append(cy * W + cx)
            n += 1
            if (cx, cy) == (sx, sy):
                return n, out, loads
            t = win[cy - y0][cx - x0]
            m = t & 0xffffffff
            if n > limit or t == EMPTY or m >= 8:
                return 0, out, loads
            cx, cy = cx - (((DXP >> (2 * m)) & 3) - 1), cy - (((DYP >> (2 * m)) & 3) - 1)
            if not (0 <= cx < W and 0 <= cy < H):
                return 0, out, loads
            if not (x0 <= cx < x0 + WIN and y0 <= cy < y0 + WIN):
                break


def _chain(rng, W, H, length):
    """A random walk of cells (no immediate repeats), start first, and a table
    whose entry at each later cell is the move from its predecessor."""
    x, y = rng.randrange(W), rng.randrange(H)
    cells = [(x, y)]
    table = [rng.choice([EMPTY, rng.randrange(1 << 40) << 8 | rng.randrange(8)]) for _ in range(W * H)]
    seen = {(x, y)}
    for _ in range(length):
        opts = [m for m in range(8) if 0 <= x + DX[m] < W and 0 <= y + DY[m] < H
                and (x + DX[m], y + DY[m]) not in seen]
        if not opts:
            break
        m = rng.choice(opts)
        x, y = x + DX[m], y + DY[m]
        seen.add((x, y))
        cells.append((x, y))
        table[y * W + x] = (rng.randrange(1 << 20) << 32) | m
    sx, sy = cells[0]
    table[sy * W + sx] = 0xff  # the start's root code
    return cells, table


@pytest.mark.parametrize("W,H", [(1, 1), (5, 3), (31, 40), (32, 32), (33, 7), (100, 64), (257, 300)])
def test_walk_returns_the_chain(W, H):
    rng = random.Random(W * 1000 + H)
    for _ in range(60):
        cells, table = _chain(rng, W, H, rng.randrange(0, 3 * (W + H)))
        start, goal = cells[0][1] * W + cells[0][0], cells[-1][1] * W + cells[-1][0]
        n, out, loads = walk(table, W, H, start, goal, limit=len(cells) + 1)
        assert n == len(cells)
        assert out == [y * W + x for x, y in reversed(cells)]
        # a short cap still counts every state
        n2, out2, _ = walk(table, W, H, start, goal, limit=len(cells) + 1, cap=3)
        assert n2 == n and out2 == out[:3]


def test_monotone_paths_take_few_loads():
    """A diagonal path toward the start crosses ~WIN - MARGIN cells per load."""
    W = H = 1000
    table = [EMPTY] * (W * H)
    for i in range(1, 900):
        table[i * W + i] = 4  # move (+1, +1) from (i-1, i-1)
    table[0] = 0xff
    n, out, loads = walk(table, W, H, 0, 899 * W + 899, limit=1000)
    assert n == 900 and loads <= 900 // (WIN - 1 - MARGIN) + 2


def test_damaged_tables_give_zero():
    W, H = 40, 40
    table = [EMPTY] * (W * H)
    table[0] = 0xff
    assert walk(table, W, H, 0, 5 * W + 5, limit=100)[0] == 0  # no move at the goal
    table[5 * W + 5] = 1  # (-1, 0) from (6, 5): leads to (6, 5), which is empty
    assert walk(table, W, H, 0, 5 * W + 5, limit=100)[0] == 0
    table[5 * W + 0] = 0  # move (+1, 0) at x = 0: its parent (-1, 5) is off the grid
    assert walk(table, W, H, 0, 5 * W, limit=100)[0] == 0
    table[3 * W + 3] = 4  # (3,3) <- (2,2) <- (3,3): a cycle, stopped by the limit
    table[2 * W + 2] = 7
    assert walk(table, W, H, 0, 3 * W + 3, limit=50)[0] == 0


def test_packed_moves_match_the_grid_domain():
    """kGridDxPack / kGridDyPack hold GridDom::dx / dy as search.cuh defines them."""
    def sets(fn):
        body = re.search(r"int %s\(int m\) \{ return ([^;]+);" % fn, SRC).group(1)
        plus, minus = re.findall(r"\(([^?]+)\) \?", body)
        return ({int(v) for v in re.findall(r"m == (\d)", plus)},
                {int(v) for v in re.findall(r"m == (\d)", minus)})
    for fn, pack, ref in (("dx", DXP, DX), ("dy", DYP, DY)):
        plus, minus = sets(fn)
        for m in range(8):
            want = 1 if m in plus else -1 if m in minus else 0
            assert ((pack >> (2 * m)) & 3) - 1 == want == ref[m], (fn, m)
