"""Grid weights reach the device by one of three paths, chosen per context
(GASTAR_UPLOAD at creation): staged (host threads copy into pinned chunks and
reduce the least passable weight while earlier chunks are sent), read in
place by a kernel that also reduces (where the GPU reads pageable host memory
through the host's page tables), or copied, then reduced.  Every path must
give numpy's least non-zero weight exactly, for buffers at every alignment,
sizes that are not multiples of 16 or of the staging chunk, grids with no
passable cell, and weight 255; and grid solves through each path must match
the oracle."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engines(gastar):
    """One engine per upload path (in place falls back to staged where the GPU
    cannot read pageable host memory)."""
    out = []
    for mode in ("staged", "inplace", "copy"):
        os.environ["GASTAR_UPLOAD"] = mode
        try:
            out.append(gastar.Engine(0))
        finally:
            del os.environ["GASTAR_UPLOAD"]
    yield out
    for e in out:
        e.close()


def _expected(w):
    nz = w[w != 0]
    return int(nz.min()) if nz.size else 255


def test_min_weight_every_path(engines, gastar):
    rng = np.random.default_rng(5)
    paths = [e.grid_min_weight(np.ones((4, 4), np.uint8))[1] for e in engines]
    assert paths[0] == "staged" and paths[2] == "copy" and paths[1] in ("inplace", "staged")
    with gastar.Engine(0) as default:  # the default path is staged
        assert default.grid_min_weight(np.ones((2, 2), np.uint8))[1] == "staged"
    shapes = [(1, 1), (3, 5), (16, 1), (17, 33), (64, 64), (1000, 1003), (2048, 2049), (4096, 4099)]
    for h, w in shapes:
        for off in (0, 1, 7, 8, 15):
            for kind in ("random", "obstacles", "heavy", "one"):
                buf = np.zeros(h * w + off, np.uint8)
                g = buf[off:].reshape(h, w)
                if kind == "random":
                    g[:] = rng.integers(0, 10, size=(h, w))
                elif kind == "obstacles":
                    g[:] = 0  # no passable cell
                elif kind == "heavy":
                    g[:] = 255
                    g[rng.integers(h), rng.integers(w)] = 0
                else:  # a single light cell somewhere in the grid
                    g[:] = rng.integers(200, 256, size=(h, w))
                    g[rng.integers(h), rng.integers(w)] = 3
                want = _expected(g)
                for eng in engines:
                    assert eng.grid_min_weight(g)[0] == want, (h, w, off, kind)


def test_grid_solves_every_path(engines, oracle, gastar):
    for i, (w, h) in enumerate([(300, 211), (1025, 999), (3001, 2999)]):
        wts = gastar.gen_grid(w, h, 9300 + i, 0.2, wmin=3)
        buf = np.zeros(w * h + 3, np.uint8)
        g = buf[3:].reshape(h, w)
        g[:] = wts
        o, _ = oracle.grid_astar(wts, (0, 0), (w - 1, h - 1), path=False)
        for eng in engines:
            r = eng.solve_grid(g, (0, 0), (w - 1, h - 1), num_queues=4096)
            assert (r.status_name, r.cost) == ("OK", o.cost)
            assert oracle.grid_validate(wts, (0, 0), (w - 1, h - 1), r.path) == (True, o.cost)
