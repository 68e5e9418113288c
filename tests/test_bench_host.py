"""Host-side pieces of bench.py that need no GPU: the CPU reference arm's
instance generator equals the engine's, and both arms print the same config."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_host_generator_matches_engine_generator(gastar):
    import bench
    for n, lo, hi in ((3, 60, 60), (4, 40, 80), (4, 20, 80), (5, 20, 40)):
        for seed in range(100):
            a = bench.gen_sliding_host(n, 7919 * seed + n, lo, hi)
            b = gastar.gen_sliding(n, 7919 * seed + n, lo, hi)
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    insts = bench._instances()
    assert len(insts) == bench.WORKLOAD["instances"]
    assert all(np.array_equal(x[0], y[0]) for x, y in zip(insts, bench._instances(gastar)))


def test_both_arms_share_the_config():
    import bench
    c = bench._config()
    assert c == bench._config() and c["workload"] == bench.WORKLOAD["name"]
    assert c["table_slots"] == 1 << bench.WORKLOAD["table_log2"]
