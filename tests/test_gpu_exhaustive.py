"""Every solvable 8-puzzle start, in batched mode, against the exhaustive BFS:
181,440 optimal costs (diameter 31).  Partitions are sized below the hardest
instances so that the overflow paths run at scale too; paths are validated
move by move on a sample."""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_all_8_puzzle_starts_batched(engine, oracle, gastar):
    goal = np.arange(9, dtype=np.uint8)
    cnt, dist = oracle.bfs8(goal)
    assert cnt == 181440
    perms = np.array(list(itertools.permutations(range(9))), dtype=np.uint8)  # index = rank
    reach = np.nonzero(dist != 255)[0]
    rng = np.random.default_rng(8)
    sample = set(rng.choice(reach, 2000, replace=False).tolist())
    chunk = 30240
    for c0 in range(0, len(reach), chunk):
        idx = reach[c0:c0 + chunk]
        b = engine.batch(warps_per_block=4, expansion_width=32, load_factor=0.75, sliding_states=8192)
        for i in idx:
            b.add_sliding(perms[i], goal)
        b.run()
        costs = np.array([b.result(j, path=False).cost for j in range(len(idx))])
        status = np.array([b.result(j, path=False).status for j in range(len(idx))])
        assert (status == gastar.OK).all()
        bad = np.nonzero(costs != dist[idx])[0]
        assert bad.size == 0, [(int(idx[k]), int(costs[k]), int(dist[idx[k]])) for k in bad[:5]]
        for j, i in enumerate(idx):
            if int(i) in sample:
                r = b.result(j, path=True)
                assert oracle.sliding_validate(3, perms[i], goal, r.path) == (True, r.cost)
        b.close()
    # The other parity class has no path; the batch answers without searching.
    b = engine.batch()
    unreach = np.nonzero(dist == 255)[0][:64]
    for i in unreach:
        b.add_sliding(perms[i], goal)
    b.run()
    assert all(b.result(j, path=False).status_name == "NO_PATH" for j in range(len(unreach)))
    b.close()
