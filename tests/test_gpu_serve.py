"""Served GA*: continuous batching gives the same results alone and in a mix."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mix(gastar, k):
    rng = np.random.default_rng(99)
    reqs = []
    for i in range(k):
        kind = i % 4
        if kind == 0:
            reqs.append(("s", *gastar.gen_sliding(3, 4000 + i, 60, 60)))
        elif kind == 1:
            reqs.append(("s", *gastar.gen_sliding(4, 4100 + i, 20, 50)))
        elif kind == 2:
            reqs.append(("s", *gastar.gen_sliding(5, 4200 + i, 10, 20)))
        else:
            side = int(rng.integers(64, 400))
            wts = gastar.gen_grid(side, side + 3, 4300 + i, 0.2)
            reqs.append(("g", wts, (0, 0), (side - 1, side + 2)))
    return reqs


def _submit(srv, r):
    return srv.submit_sliding(r[1], r[2]) if r[0] == "s" else srv.submit_grid(r[1], r[2], r[3])


def _check(oracle, r, res):
    if r[0] == "s":
        n = int(round(len(r[1]) ** 0.5))
        o, _ = oracle.sliding_astar(n, r[1], r[2], path=False)
        assert res.status_name == "OK" and res.cost == o.cost
        assert oracle.sliding_validate(n, r[1], r[2], res.path) == (True, res.cost)
    else:
        o, _ = oracle.grid_astar(r[1], r[2], r[3], path=False)
        assert res.status_name == "OK" and res.cost == o.cost
        assert oracle.grid_validate(r[1], r[2], r[3], res.path) == (True, res.cost)


@pytest.mark.parametrize("open_list", [0, 1])
def test_results_same_alone_and_in_mix(engine, oracle, gastar, open_list):
    """Requests suspended every 16 iterations (heaps, or buckets whose state is
    kept beside their pages) match the oracle, alone and in the mix."""
    reqs = _mix(gastar, 24)
    srv = engine.server(slice_iters=16, budget_bytes=8 << 30, open_list=open_list)
    # Staggered arrivals: a third before the first step, the rest while running.
    ids = [_submit(srv, r) for r in reqs[:8]]
    srv.step()
    ids += [_submit(srv, r) for r in reqs[8:16]]
    srv.step()
    ids += [_submit(srv, r) for r in reqs[16:]]
    mixed = srv.drain(ids)
    srv.close()
    for r, i in zip(reqs, ids):
        _check(oracle, r, mixed[i])
    # The same requests one at a time.
    for r, i in zip(reqs, ids):
        one = engine.server(slice_iters=16, budget_bytes=2 << 30, open_list=open_list)
        j = _submit(one, r)
        alone = one.drain([j])[j]
        one.close()
        assert (alone.status, alone.cost) == (mixed[i].status, mixed[i].cost)


def test_budget_limits_admission(engine, oracle, gastar):
    """A small budget admits few requests at a time; all still finish."""
    srv = engine.server(slice_iters=32, budget_bytes=256 << 20)
    reqs = [("s", *gastar.gen_sliding(4, 5000 + i, 20, 40)) for i in range(12)]
    ids = [_submit(srv, r) for r in reqs]
    srv.step()
    st = srv.stats()
    assert st["active"] < 12 and st["waiting"] > 0
    out = srv.drain(ids)
    for r, i in zip(reqs, ids):
        _check(oracle, r, out[i])
    srv.close()


def test_served_mix_at_benchmark_sizes(engine, oracle, gastar):
    """Requests at the served benchmark's own sizes -- 8-puzzles (walk 60),
    15-puzzles (walk 20-80), 24-puzzles (walk 20-40, 128-bit keys) and grids
    of side 512-5000 (the larger ones heavy, on multi-block teams) -- arriving
    while the server runs under its default configuration: every cost equals
    the oracle's and every path is valid."""
    reqs = [("s", *gastar.gen_sliding(3, 6000 + i, 60, 60)) for i in range(4)]
    reqs += [("s", *gastar.gen_sliding(4, 6100 + i, 20, 80)) for i in range(6)]
    reqs += [("s", *gastar.gen_sliding(5, 6200 + i, 20, 40)) for i in range(4)]
    for i, side in enumerate((512, 1500, 3000, 5000)):
        reqs.append(("g", gastar.gen_grid(side, side, 6300 + i, 0.2), (0, 0), (side - 1, side - 1)))
    order = np.random.default_rng(6400).permutation(len(reqs))
    srv = engine.server(budget_bytes=64 << 30)
    ids = {}
    for k, j in enumerate(order):
        ids[int(j)] = _submit(srv, reqs[j])
        if k % 3 == 2:
            srv.step()
    out = srv.drain(list(ids.values()))
    srv.close()
    gi = [j for j, r in enumerate(reqs) if r[0] == "g"]
    _, ref_g = oracle.grid_batch([reqs[j][1:] for j in gi])
    for j, o in zip(gi, ref_g):
        r, res = reqs[j], out[ids[j]]
        assert res.status_name == "OK" and res.cost == o.cost
        assert oracle.grid_validate(r[1], r[2], r[3], res.path) == (True, res.cost)
    for j, r in enumerate(reqs):
        if r[0] == "s":
            _check(oracle, r, out[ids[j]])


def test_hard_puzzles_promoted_to_the_plain_engine(engine, oracle, gastar):
    """With a low promotion budget (2^12 expansions) most 15- and 24-puzzle
    requests leave their slot mid-search and are finished by the plain engine
    between two steps; grids and 8-puzzles stay; every result matches the
    oracle, paths included."""
    reqs = [("s", *gastar.gen_sliding(4, 6500 + i, 30, 60)) for i in range(6)]
    reqs += [("s", *gastar.gen_sliding(5, 6600 + i, 16, 24)) for i in range(2)]
    reqs += [("s", *gastar.gen_sliding(3, 6700 + i, 60, 60)) for i in range(2)]
    reqs.append(("g", gastar.gen_grid(300, 280, 6800, 0.2), (0, 0), (299, 279)))
    srv = engine.server(slice_iters=16, budget_bytes=8 << 30, promote_log2=12)
    ids = [_submit(srv, r) for r in reqs]
    out = srv.drain(ids)
    srv.close()
    for r, i in zip(reqs, ids):
        _check(oracle, r, out[i])
    # at least the 15-puzzles passed 2^12 expansions (and were promoted)
    assert sum(out[i].expansions > (1 << 12) for i in ids[:6]) >= 3


def test_grid_weights_in_the_pool_and_host_copies(engine, oracle, gastar):
    """Grid weights go from the caller's buffer to the device pool at
    submission (an eighth of the budget: 32 MiB here); once 32 grids of 1 MB
    fill it, later ones keep a host copy sent at admission.  Both kinds match
    the oracle, and a server without a pool returns the same costs."""
    reqs = []
    for i in range(40):
        w, h = 1000 + (i % 3), 1000 + (i % 5)
        reqs.append(("g", gastar.gen_grid(w, h, 7000 + i, 0.2), (0, 0), (w - 1, h - 1)))
    res = {}
    for pool in (1, 0):
        srv = engine.server(budget_bytes=256 << 20, slice_iters=32, weights_pool=pool)
        ids = [_submit(srv, r) for r in reqs]
        out = srv.drain(ids)
        srv.close()
        res[pool] = [out[i] for i in ids]
        for k, r in enumerate(reqs):
            # every grid's weights arrays may be reused by the caller now
            assert res[pool][k].status_name == "OK"
    _, ref = oracle.grid_batch([r[1:] for r in reqs])
    for k, (r, o) in enumerate(zip(reqs, ref)):
        assert res[1][k].cost == res[0][k].cost == o.cost
        assert oracle.grid_validate(r[1], r[2], r[3], res[1][k].path) == (True, o.cost)


def test_small_requests_pass_a_large_one_waiting_for_memory(engine, oracle, gastar):
    """20 grids of 3000^2 need more than the 4 GiB budget, so some wait for
    memory; 64^2 grids submitted after them (partitions under 1/256 of the
    budget) are admitted at once with admit_bypass, and wait behind the
    large ones in strict arrival order.  Results are the same either way."""
    big = [("g", gastar.gen_grid(3000, 3000, 7100 + i, 0.2), (0, 0), (2999, 2999)) for i in range(20)]
    small = [("g", gastar.gen_grid(64, 64, 7200 + i, 0.2), (0, 0), (63, 63)) for i in range(8)]
    waiting, res = {}, {}
    for bypass in (1, 0):
        srv = engine.server(budget_bytes=4 << 30, admit_bypass=bypass)
        ids = [_submit(srv, r) for r in big + small]
        srv.step()
        waiting[bypass] = srv.stats()["waiting"]
        out = srv.drain(ids)
        srv.close()
        res[bypass] = [out[i] for i in ids]
    assert waiting[1] >= 1  # a large grid waits for memory
    assert waiting[0] == waiting[1] + len(small)
    assert [(r.status, r.cost) for r in res[1]] == [(r.status, r.cost) for r in res[0]]
    for k, r in enumerate(small):
        _check(oracle, r, res[1][len(big) + k])
