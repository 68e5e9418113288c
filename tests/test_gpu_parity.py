"""GPU engine against the CPU oracle through the C ABI (plain GA*)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check_sliding(oracle, n, s, g, r, heuristic=0, ref_moves=0):
    o, _ = oracle.sliding_astar(n, s, g, heuristic=heuristic, ref_moves=ref_moves, path=False)
    if o.status == oracle.NO_PATH:
        assert r.status_name == "NO_PATH"
        return o
    assert r.status_name == "OK", r
    if heuristic == 0:
        assert r.cost == o.cost
    else:  # an inadmissible heuristic: valid path, never below the optimum (admissible A*)
        opt, _ = oracle.sliding_astar(n, s, g, heuristic=0, ref_moves=ref_moves, path=False)
        assert r.cost >= opt.cost
    ok, cost = oracle.sliding_validate(n, s, g, r.path, ref_moves=ref_moves)
    assert ok and cost == r.cost and len(r.path) == r.cost + 1
    return o


def test_8_puzzle_against_bfs(engine, oracle, gastar):
    goal = np.arange(9, dtype=np.uint8)
    _, dist = oracle.bfs8(goal)
    rng = np.random.default_rng(11)
    for i in range(40):
        s = rng.permutation(9).astype(np.uint8)
        d = dist[oracle.perm_rank9(s)]
        r = engine.solve_sliding(s, goal, 3, num_queues=256)
        if d == 255:
            assert r.status_name == "NO_PATH"
            continue
        assert r.status_name == "OK" and r.cost == d, (i, r.status_name, r.cost, d)
        ok, cost = oracle.sliding_validate(3, s, goal, r.path)
        assert ok and cost == d


@pytest.mark.parametrize("queues", [32, 1024, 16384])
def test_15_puzzle_random_walks(engine, oracle, gastar, queues):
    for seed in range(6):
        s, g = gastar.gen_sliding(4, 1000 + seed, 30, 60)
        r = engine.solve_sliding(s, g, 4, num_queues=queues)
        _check_sliding(oracle, 4, s, g, r)


def test_24_puzzle_short_walks(engine, oracle, gastar):
    for seed in range(4):
        s, g = gastar.gen_sliding(5, 2000 + seed, 14, 26)
        r = engine.solve_sliding(s, g, 5, num_queues=2048)
        _check_sliding(oracle, 5, s, g, r)


def test_reference_heuristic_and_moves(engine, oracle, gastar):
    for seed in range(4):
        s, g = gastar.gen_sliding(4, 3000 + seed, 20, 40)
        r = engine.solve_sliding(s, g, 4, num_queues=1024, heuristic=gastar.H_REFERENCE)
        _check_sliding(oracle, 4, s, g, r, heuristic=1)
    goal = np.arange(9, dtype=np.uint8)
    ok, _, one = oracle.sliding_successor(3, goal, 0, 1)
    ok2, _, two = oracle.sliding_successor(3, one, 2, 1)
    r = engine.solve_sliding(goal, two, 3, moves=gastar.MOVES_REFERENCE)
    assert r.status_name == "OK" and r.cost == 2
    assert oracle.sliding_validate(3, goal, two, r.path, ref_moves=1) == (True, 2)
    r = engine.solve_sliding(two, goal, 3, moves=gastar.MOVES_REFERENCE)
    assert r.status_name == "NO_PATH"


def test_sliding_edge_cases(engine, oracle, gastar):
    goal = np.arange(16, dtype=np.uint8)
    r = engine.solve_sliding(goal, goal, 4)
    assert r.status_name == "OK" and r.cost == 0 and len(r.path) == 1
    bad = goal.copy()
    bad[[1, 2]] = bad[[2, 1]]
    r = engine.solve_sliding(bad, goal, 4)
    assert r.status_name == "NO_PATH" and r.expansions == 0
    with pytest.raises(gastar.GastarError):
        engine.solve_sliding(np.zeros(16, np.uint8), goal, 4)
    s, g = gastar.gen_sliding(4, 77, 60, 60)
    r = engine.solve_sliding(s, g, 4, num_queues=256, max_expansions=50, regrow=0)
    assert r.status_name == "BUDGET"


def test_device_deadline_and_heap_capacity(engine, oracle, gastar):
    """Limits end a search with a status and leave the context usable."""
    s, g = gastar.gen_sliding(5, 6000, 60, 60)      # far beyond 1 ms of search
    r = engine.solve_sliding(s, g, 5, num_queues=1024, timeout_ms=1, table_log2=26, regrow=0,
                             path=False)
    assert r.status_name == "TIMEOUT"
    s2, g2 = gastar.gen_sliding(4, 6001, 20, 30)
    _check_sliding(oracle, 4, s2, g2, engine.solve_sliding(s2, g2, 4, num_queues=4096))
    s3, g3 = gastar.gen_sliding(4, 6002, 80, 80)    # open list far above 8 small heaps
    r = engine.solve_sliding(s3, g3, 4, num_queues=64, heap_entries=64, regrow=0, path=False)
    assert r.status_name == "HEAP_FULL"
    _check_sliding(oracle, 4, s2, g2, engine.solve_sliding(s2, g2, 4, num_queues=4096))


def test_table_regrow(engine, oracle, gastar):
    s, g = gastar.gen_sliding(4, 4242, 50, 50)
    cfg = gastar.make_config(num_queues=512, table_log2=10)
    r = engine.solve_sliding(s, g, 4, config=cfg)
    assert r.attempts > 1
    _check_sliding(oracle, 4, s, g, r)


@pytest.mark.parametrize("open_list", [0, 1])
def test_open_list_modes(engine, oracle, gastar, open_list):
    """Warp-heaps alone (0) and shared-memory f-buckets in front of them (1)
    give the same optimal costs, one block and multi-block teams."""
    for seed, queues in ((0, 32), (1, 4096), (2, 16384)):
        s, g = gastar.gen_sliding(4, 5000 + seed, 40, 70)
        r = engine.solve_sliding(s, g, 4, num_queues=queues, open_list=open_list)
        _check_sliding(oracle, 4, s, g, r)
    s, g = gastar.gen_sliding(5, 5100, 16, 24)
    r = engine.solve_sliding(s, g, 5, num_queues=4096, open_list=open_list)
    _check_sliding(oracle, 5, s, g, r)
    wts = gastar.gen_grid(257, 193, 5200, 0.25)
    for queues in (64, 8192):
        r = engine.solve_grid(wts, (3, 2), (250, 190), num_queues=queues, open_list=open_list)
        _check_grid(oracle, wts, (3, 2), (250, 190), r)


def _check_grid(oracle, wts, st, gl, r):
    o, _ = oracle.grid_astar(wts, st, gl, path=False)
    if o.status == oracle.NO_PATH:
        assert r.status_name == "NO_PATH"
        return
    assert r.status_name == "OK" and r.cost == o.cost, (r.status_name, r.cost, o.cost)
    ok, cost = oracle.grid_validate(wts, st, gl, r.path)
    assert ok and cost == r.cost


@pytest.mark.parametrize("queues", [64, 4096, 65536])
def test_grids_against_oracle(engine, oracle, gastar, queues):
    rng = np.random.default_rng(5)
    for t in range(5):
        w, h = int(rng.integers(2, 300)), int(rng.integers(2, 300))
        wts = gastar.gen_grid(w, h, 50 + t, float(rng.uniform(0.1, 0.3)))
        st, gl = (0, 0), (w - 1, h - 1)
        r = engine.solve_grid(wts, st, gl, num_queues=queues)
        _check_grid(oracle, wts, st, gl, r)
        st2 = (int(rng.integers(0, w)), int(rng.integers(0, h)))
        r = engine.solve_grid(wts, st2, gl, num_queues=queues)
        _check_grid(oracle, wts, st2, gl, r)


def test_grid_edge_cases(engine, oracle, gastar):
    one = np.ones((1, 1), np.uint8)
    r = engine.solve_grid(one, (0, 0), (0, 0))
    assert r.status_name == "OK" and r.cost == 0
    wts = np.ones((5, 5), np.uint8)
    wts[:, 2] = 0
    r = engine.solve_grid(wts, (0, 0), (4, 4))
    assert r.status_name == "NO_PATH"
    wts = np.ones((5, 5), np.uint8)
    wts[4, 4] = 0
    assert engine.solve_grid(wts, (0, 0), (4, 4)).status_name == "NO_PATH"
    wts[0, 0] = 0   # an impassable start is still expanded
    r = engine.solve_grid(wts, (0, 0), (3, 3))
    _check_grid(oracle, wts, (0, 0), (3, 3), r)
    wts = gastar.gen_grid(200, 120, 3, 0.2)
    for heur in (gastar.H_REFERENCE, gastar.H_ZERO):
        r = engine.solve_grid(wts, (0, 0), (199, 119), heuristic=heur)
        o, _ = oracle.grid_astar(wts, (0, 0), (199, 119), heuristic=heur, path=False)
        ok, cost = oracle.grid_validate(wts, (0, 0), (199, 119), r.path)
        assert r.status_name == "OK" and ok and cost == r.cost
        if heur == gastar.H_ZERO:
            assert r.cost == o.cost


@pytest.mark.parametrize("delta", [36, 0])
def test_4096_grid_full_size(engine, oracle, gastar, delta):
    """The plain grid configuration at full size: 4096 x 4096, weights 1..9,
    20 % obstacles, a monotone corridor from (0, 0) to (4095, 4095); optimal
    cost equal to the oracle's and a valid path (with and without the pop
    window)."""
    wts = gastar.gen_grid(4096, 4096, 0x4096, 0.2)
    r = engine.solve_grid(wts, (0, 0), (4095, 4095), num_queues=16384, delta=delta)
    _check_grid(oracle, wts, (0, 0), (4095, 4095), r)
    assert len(r.path) > 4095 and r.path[0] == 0 and r.path[-1] == 4096 * 4096 - 1


def test_widened_pops_on_the_hardest_benchmark_puzzles(engine, oracle, gastar):
    """The plain benchmark's three hardest 15-puzzles (seeds 0x150000 + 38,
    17, 31 of its walk 40-80 set) run for hundreds of iterations at Q = 16384:
    past the 64th the automatic width doubles every warp-heap's pops.  Costs
    equal the oracle's and paths are valid, widened and at a fixed width."""
    insts = [gastar.gen_sliding(4, 0x15_0000 + i, 40, 80) for i in (38, 17, 31)]
    _, ref = oracle.sliding_batch(4, np.stack([s for s, _ in insts]), np.stack([g for _, g in insts]))
    for (s, g), o in zip(insts, ref):
        wide = engine.solve_sliding(s, g, 4, num_queues=16384, table_log2=30)
        assert wide.iterations > 64  # the widened iterations ran
        fixed = engine.solve_sliding(s, g, 4, num_queues=16384, table_log2=30, expansion_width=16)
        for r in (wide, fixed):
            assert r.status_name == "OK" and r.cost == o.cost
            assert oracle.sliding_validate(4, s, g, r.path) == (True, r.cost)
        assert wide.iterations < fixed.iterations
