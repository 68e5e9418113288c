"""The oracle's A* pinned by independent exhaustive searches (CPU only)."""
import numpy as np
import pytest


def _rand_board(rng, n):
    return rng.permutation(n * n).astype(np.uint8)


def test_bfs8_known_facts(oracle):
    goal = np.arange(9, dtype=np.uint8)
    count, dist = oracle.bfs8(goal)
    assert count == 181440                     # half of 9! is reachable
    assert int(dist[dist != 255].max()) == 31  # 8-puzzle diameter


@pytest.mark.parametrize("goal_seed", [0, 1])
def test_astar_matches_bfs_on_8_puzzle(oracle, goal_seed):
    rng = np.random.default_rng(100 + goal_seed)
    goal = np.arange(9, dtype=np.uint8) if goal_seed == 0 else _rand_board(rng, 3)
    _, dist = oracle.bfs8(goal)
    for _ in range(300):
        s = _rand_board(rng, 3)
        d = dist[oracle.perm_rank9(s)]
        r, p = oracle.sliding_astar(3, s, goal)
        if d == 255:
            assert not oracle.sliding_solvable(3, s, goal)
            continue
        assert r.status == oracle.OK and r.cost == d
        ok, cost = oracle.sliding_validate(3, s, goal, p)
        assert ok and cost == d
        # Dijkstra order reaches the same optimum
        r0, _ = oracle.sliding_astar(3, s, goal, heuristic=oracle.ZERO, path=False)
        assert r0.cost == d


def test_unsolvable_8_puzzle_exhausts(oracle):
    goal = np.arange(9, dtype=np.uint8)
    s = goal.copy()
    s[[1, 2]] = s[[2, 1]]
    assert not oracle.sliding_solvable(3, s, goal)
    r, _ = oracle.sliding_astar(3, s, goal, path=False)
    assert r.status == oracle.NO_PATH and r.expansions == 181440


def test_reference_moves_reach_only_down_right(oracle):
    goal = np.arange(9, dtype=np.uint8)          # blank at (0,0)
    ok, _, one = oracle.sliding_successor(3, goal, 2, ref_moves=1)  # blank right
    assert ok
    r, p = oracle.sliding_astar(3, goal, one, ref_moves=1)
    assert r.status == oracle.OK and r.cost == 1
    r, _ = oracle.sliding_astar(3, one, goal, ref_moves=1, path=False)  # needs a col-1 move
    assert r.status == oracle.NO_PATH


def _dijkstra(wts, start, goal):
    import heapq
    h, w = wts.shape
    dist = np.full((h, w), np.iinfo(np.int64).max, dtype=np.int64)
    dist[start[1], start[0]] = 0
    pq = [(0, start[0], start[1])]
    while pq:
        d, x, y = heapq.heappop(pq)
        if d > dist[y, x]:
            continue
        if (x, y) == tuple(goal):
            return d
        for dx, dy in ((1, 0), (-1, 0), (0, 1), (0, -1), (1, 1), (1, -1), (-1, 1), (-1, -1)):
            nx, ny = x + dx, y + dy
            if 0 <= nx < w and 0 <= ny < h and wts[ny, nx]:
                nd = d + int(wts[ny, nx])
                if nd < dist[ny, nx]:
                    dist[ny, nx] = nd
                    heapq.heappush(pq, (nd, nx, ny))
    return None


def test_grid_astar_matches_dijkstra(oracle):
    rng = np.random.default_rng(7)
    for t in range(60):
        w, h = int(rng.integers(1, 40)), int(rng.integers(1, 40))
        wts = rng.integers(1, 10, size=(h, w)).astype(np.uint8)
        wts[rng.random((h, w)) < rng.uniform(0, 0.45)] = 0
        st = (int(rng.integers(0, w)), int(rng.integers(0, h)))
        gl = (int(rng.integers(0, w)), int(rng.integers(0, h)))
        ref = _dijkstra(wts, st, gl)
        for heur in (oracle.ADM, oracle.ZERO):
            r, p = oracle.grid_astar(wts, st, gl, heuristic=heur)
            if ref is None:
                assert r.status == oracle.NO_PATH
            else:
                assert r.status == oracle.OK and r.cost == ref, (t, heur)
                ok, cost = oracle.grid_validate(wts, st, gl, p)
                assert ok and cost == ref


def test_validators_reject_bad_paths(oracle):
    goal = np.arange(9, dtype=np.uint8)
    s = goal.copy()
    s[[0, 1]] = s[[1, 0]]  # one move away
    r, p = oracle.sliding_astar(3, s, goal)
    assert oracle.sliding_validate(3, s, goal, p) == (True, 1)
    bad = p.copy()
    bad[1] = bad[0]
    assert not oracle.sliding_validate(3, s, goal, bad)[0]
    wts = np.ones((3, 3), np.uint8)
    assert oracle.grid_validate(wts, (0, 0), (2, 2), [0, 4, 8]) == (True, 2)
    assert not oracle.grid_validate(wts, (0, 0), (2, 2), [0, 8])[0]        # jump
    wts[1, 1] = 0
    assert not oracle.grid_validate(wts, (0, 0), (2, 2), [0, 4, 8])[0]     # obstacle


def test_batch_threads_agree_with_single(oracle):
    rng = np.random.default_rng(3)
    goal = np.arange(9, dtype=np.uint8)
    starts = [_rand_board(rng, 3) for _ in range(16)]
    used, res = oracle.sliding_batch(3, starts, [goal] * 16, threads=4)
    assert used == 4
    for s, r in zip(starts, res):
        single, _ = oracle.sliding_astar(3, s, goal, path=False)
        assert (r.status, r.cost) == (single.status, single.cost)
