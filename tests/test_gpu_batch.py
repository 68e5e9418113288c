"""Batched GA* (one persistent launch) against the oracle and the plain engine."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("open_list", [0, 1])
def test_mixed_batch_matches_oracle(engine, oracle, gastar, open_list):
    b = engine.batch(warps_per_block=8, expansion_width=32, open_list=open_list)
    cases = []
    for i in range(24):
        s, g = gastar.gen_sliding(4, 500 + i, 20, 50)
        cases.append(("s4", s, g, b.add_sliding(s, g)))
    for i in range(8):
        s, g = gastar.gen_sliding(3, 600 + i, 60, 60)
        cases.append(("s3", s, g, b.add_sliding(s, g)))
    for i in range(3):
        s, g = gastar.gen_sliding(5, 700 + i, 10, 20)
        cases.append(("s5", s, g, b.add_sliding(s, g)))
    for i in range(12):
        side = 40 + 23 * i
        wts = gastar.gen_grid(side, side + 7, 800 + i, 0.2)
        cases.append(("grid", wts, ((0, 0), (side - 1, side + 6)), b.add_grid(wts, (0, 0), (side - 1, side + 6))))
    bad = np.arange(16, dtype=np.uint8)
    bad[[1, 2]] = bad[[2, 1]]
    cases.append(("bad", bad, np.arange(16, dtype=np.uint8), b.add_sliding(bad, np.arange(16, dtype=np.uint8))))
    b.run()
    for kind, a, c, idx in cases:
        r = b.result(idx)
        if kind == "bad":
            assert r.status_name == "NO_PATH"
            continue
        if kind == "grid":
            st, gl = c
            o, _ = oracle.grid_astar(a, st, gl, path=False)
            assert r.status_name == "OK" and r.cost == o.cost, (idx, r.status_name)
            assert oracle.grid_validate(a, st, gl, r.path) == (True, r.cost)
        else:
            n = {"s3": 3, "s4": 4, "s5": 5}[kind]
            o, _ = oracle.sliding_astar(n, a, c, path=False)
            assert r.status_name == "OK" and r.cost == o.cost, (idx, kind, r.status_name, r.cost, o.cost)
            assert oracle.sliding_validate(n, a, c, r.path) == (True, r.cost)
    costs = [b.result(i, path=False).cost for _, _, _, i in cases]
    b.rerun()   # inputs stay resident; graph replay
    assert [b.result(i, path=False).cost for _, _, _, i in cases] == costs
    st = b.stats()
    assert st["kernel_ms"] > 0 and st["device_bytes"] > 0
    # The launch's schedule: every solved instance ran inside the launch,
    # the unreachable board never started.
    t0, t1 = b.timeline()
    bad_idx = cases[-1][3]
    assert t0[bad_idx] == 0 and t1[bad_idx] == 0
    ran = [i for _, _, _, i in cases if i != bad_idx]
    assert all(t1[i] >= t0[i] for i in ran) and min(t0[i] for i in ran) == 0
    assert max(t1[i] for i in ran) <= (st["main_ms"] + 1.0) * 1e6
    b.close()


def test_batch_equals_plain(engine, gastar):
    b = engine.batch(warps_per_block=4, expansion_width=16)
    inst = [gastar.gen_sliding(4, 900 + i, 30, 60) for i in range(8)]
    for s, g in inst:
        b.add_sliding(s, g)
    b.run()
    for i, (s, g) in enumerate(inst):
        assert b.result(i, path=False).cost == engine.solve_sliding(s, g, 4, path=False).cost
    b.close()


@pytest.mark.parametrize("count", [6, 70])
def test_batch_partition_overflow_is_retried(engine, oracle, gastar, count):
    """Partitions sized far below the need overflow.  A few overflowed
    instances are re-solved by the plain engine; many go through a second
    batch launch with larger partitions first.  All still match the oracle."""
    b = engine.batch(warps_per_block=4, expansion_width=32, load_factor=0.75, sliding_states=256)
    inst = [gastar.gen_sliding(4, 1300 + i, 25, 40) for i in range(count)]
    for s, g in inst:
        b.add_sliding(s, g)
    b.run()
    st = b.stats()
    if count <= 64:
        assert st["retried"] == 0 and st["promoted"] > 0
    else:
        assert st["retried"] > 64
    for i, (s, g) in enumerate(inst):
        r = b.result(i)
        o, _ = oracle.sliding_astar(4, s, g, path=False)
        assert r.status_name == "OK" and r.cost == o.cost
        assert oracle.sliding_validate(4, s, g, r.path) == (True, r.cost)
    b.rerun()  # the kept re-run batch is replayed
    assert b.stats()["retried"] == st["retried"]
    for i, (s, g) in enumerate(inst):
        r = b.result(i)
        o, _ = oracle.sliding_astar(4, s, g, path=False)
        assert r.status_name == "OK" and r.cost == o.cost
        assert oracle.sliding_validate(4, s, g, r.path) == (True, r.cost)
    b.close()


def test_heavy_teams_and_promotion(engine, oracle, gastar):
    """Large grids run on multi-block teams, and a puzzle past its expansion
    budget is re-solved by the plain engine; all results match the oracle."""
    b = engine.batch(warps_per_block=4, expansion_width=32, heavy_team=2, heavy_cells=200 * 200,
                     promote_expansions=2000)
    cases = []
    for i in range(6):
        side = 180 + 40 * i
        wts = gastar.gen_grid(side, side, 1400 + i, 0.2)
        cases.append(("g", wts, b.add_grid(wts, (0, 0), (side - 1, side - 1)), side))
    for i in range(6):
        s, g = gastar.gen_sliding(4, 1500 + i, 30, 50)
        cases.append(("s", (s, g), b.add_sliding(s, g), 0))
    b.run()
    for kind, a, idx, side in cases:
        r = b.result(idx)
        if kind == "g":
            o, _ = oracle.grid_astar(a, (0, 0), (side - 1, side - 1), path=False)
            assert r.status_name == "OK" and r.cost == o.cost
            assert oracle.grid_validate(a, (0, 0), (side - 1, side - 1), r.path) == (True, r.cost)
        else:
            s, g = a
            o, _ = oracle.sliding_astar(4, s, g, path=False)
            assert r.status_name == "OK" and r.cost == o.cost
            assert oracle.sliding_validate(4, s, g, r.path) == (True, r.cost)
    b.rerun()
    for kind, a, idx, side in cases:
        assert b.result(idx, path=False).status_name == "OK"
    b.close()


def test_config_b_shape_against_oracle(engine, oracle, gastar):
    """A stratified sample of the 1024-instance batched mix at its own sizes:
    15-puzzles with walks 20-80 (the hard ones pass the promotion budget and
    are re-solved by the plain engine) and grids of side 256-2048 with obstacle
    density 0.1-0.3 (the largest on two-block teams), under the autotuner's
    usual pick.  Every cost equals the oracle's and every path is valid, on
    the first run and on two device-resident re-runs, which clear only the
    table slots the previous search claimed."""
    seed0 = 0x3_0000  # the batched mix of the benchmark
    rng = np.random.default_rng(seed0)
    sides, dens = [], []
    for _ in range(512):  # the benchmark's draw order: side, then density, per grid
        sides.append(int(rng.integers(256, 2049)))
        dens.append(float(rng.uniform(0.1, 0.3)))
    b = engine.batch(warps_per_block=16, expansion_width=32, load_factor=0.5, delta_grid=18,
                     heavy_team=2, heavy_cells=1 << 21, open_list=1)
    puzzles = [gastar.gen_sliding(4, seed0 + i, 20, 80) for i in range(0, 512, 8)]
    order = sorted(range(512), key=lambda i: sides[i])
    picks = order[::32] + order[-2:]  # sides across the range, the two largest included
    grids = [(gastar.gen_grid(sides[i], sides[i], seed0 + 100_000 + i, dens[i]), sides[i]) for i in picks]
    for s, g in puzzles:
        b.add_sliding(s, g)
    for w, side in grids:
        b.add_grid(w, (0, 0), (side - 1, side - 1))
    _, ref_p = oracle.sliding_batch(4, np.stack([s for s, _ in puzzles]), np.stack([g for _, g in puzzles]))
    _, ref_g = oracle.grid_batch([(w, (0, 0), (side - 1, side - 1)) for w, side in grids])
    want = [r.cost for r in ref_p] + [r.cost for r in ref_g]
    b.run()
    assert b.stats()["promoted"] > 0  # the plain-engine re-solve path ran
    for run in range(3):
        if run:
            b.rerun()
        res = [b.result(i, path=True) for i in range(len(b))]
        assert [r.status_name for r in res] == ["OK"] * len(res)
        assert [r.cost for r in res] == want, run
        for i, (s, g) in enumerate(puzzles):
            assert oracle.sliding_validate(4, s, g, res[i].path) == (True, want[i])
        for j, (w, side) in enumerate(grids):
            k = len(puzzles) + j
            assert oracle.grid_validate(w, (0, 0), (side - 1, side - 1), res[k].path) == (True, want[k])
    b.close()
