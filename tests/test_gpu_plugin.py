"""The generic template API (reference plugin types on the engine), the
reference-compatible solve() front ends and the astar_gpu command on a GPU."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "cuda_a_star_gb300", "_build", "astar_gpu")


@pytest.fixture(scope="module")
def harness(gastar):
    sys.path.insert(0, os.path.join(ROOT, "tests", "plugin"))
    import build_harness
    lib = C.CDLL(build_harness.build())
    u8, u32 = C.POINTER(C.c_uint8), C.POINTER(C.c_uint32)
    lib.harness_sliding.argtypes = [C.c_uint32, u8, u8, C.c_uint32, C.c_int, u8]
    lib.harness_grid.argtypes = [C.c_uint32, C.c_uint32, u8, C.c_uint32, C.c_uint32, C.c_uint32,
                                 C.c_uint32, C.c_uint32, u32]
    lib.harness_line.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, u32]
    lib.harness_solve_text.argtypes = [C.c_int, C.c_uint32, C.c_char_p, C.c_uint32, C.c_char_p,
                                       C.c_size_t]
    return lib


def _u8(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint8))


@pytest.mark.parametrize("n,walk", [(3, (40, 60)), (4, (20, 40)), (5, (10, 20))])
def test_reference_plugin_types_on_template_api(harness, oracle, gastar, n, walk):
    for seed in range(3):
        s, g = gastar.gen_sliding(n, 7000 + 10 * n + seed, *walk)
        out = np.zeros((512, n * n), np.uint8)
        ln = harness.harness_sliding(n, _u8(s), _u8(g), 2048, 0, _u8(out))
        o, _ = oracle.sliding_astar(n, s, g, path=False)
        assert ln == o.cost + 1
        assert oracle.sliding_validate(n, s, g, out[:ln]) == (True, o.cost)
    # the reference's own (inadmissible) heuristic still yields a valid path
    s, g = gastar.gen_sliding(n, 7100 + n, *walk)
    out = np.zeros((2048, n * n), np.uint8)
    ln = harness.harness_sliding(n, _u8(s), _u8(g), 2048, 1, _u8(out))
    o, _ = oracle.sliding_astar(n, s, g, path=False)
    ok, cost = oracle.sliding_validate(n, s, g, out[:ln])
    assert ok and cost >= o.cost


def test_grid_plugin_on_template_api(harness, oracle, gastar):
    for seed in range(3):
        w, h = 90 + 30 * seed, 70
        wts = gastar.gen_grid(w, h, 7200 + seed, 0.2)
        out = np.zeros(w * h, np.uint32)
        ln = harness.harness_grid(w, h, _u8(wts), 0, 0, w - 1, h - 1, 4096,
                                  out.ctypes.data_as(C.POINTER(C.c_uint32)))
        o, _ = oracle.grid_astar(wts, (0, 0), (w - 1, h - 1), path=False)
        assert oracle.grid_validate(wts, (0, 0), (w - 1, h - 1), out[:ln]) == (True, o.cost)


def _line_dijkstra(limit, start, target):
    import heapq
    dist = {start: 0}
    pq = [(0, start)]
    while pq:
        d, v = heapq.heappop(pq)
        if v == target:
            return d
        if d > dist[v]:
            continue
        for nv, c in ((v + 1, 1), (v - 1, 1), (v * 2, 3)):
            if 0 <= nv < limit and (nv != v * 2 or v * 2 < limit) and d + c < dist.get(nv, 1 << 60):
                dist[nv] = d + c
                heapq.heappush(pq, (d + c, nv))
    return None


def test_custom_plugin_without_reference_counterpart(harness):
    for start, target in ((3, 1000), (999, 2), (0, 4095), (17, 17)):
        out = np.zeros(8192, np.uint32)
        ln = harness.harness_line(5000, start, target, 512, out.ctypes.data_as(C.POINTER(C.c_uint32)))
        path = out[:ln].tolist()
        assert path[0] == start and path[-1] == target
        cost = 0
        for a, b in zip(path, path[1:]):
            assert b in (a + 1, a - 1, 2 * a)
            cost += 1 if abs(b - a) == 1 else 3   # 1 -> 2 is the cheaper +1 step
        assert cost == _line_dijkstra(5000, start, target)


def test_reference_solve_front_ends(harness, oracle, gastar):
    s, g = gastar.gen_sliding(4, 7300, 30, 50)
    text = f"{gastar.format_sliding(s)} {gastar.format_sliding(g)}"
    buf = C.create_string_buffer(1 << 16)
    ln = harness.harness_solve_text(0, 4, text.encode(), 4096, buf, len(buf))
    lines = buf.value.decode().split()
    path = np.array([[0 if t == "_" else int(t) for t in l.split(",")] for l in lines], np.uint8)
    o, _ = oracle.sliding_astar(4, s, g, path=False)
    assert ln > 0 and oracle.sliding_validate(4, s, g, path) == (True, o.cost)
    doc = "6,5\n0,0\n5,4\n3\n1,1\n2,2\n3,3\n2\n4,3,7\n1,3,2\n"
    ln = harness.harness_solve_text(1, 0, doc.encode(), 4096, buf, len(buf))
    cells = [tuple(map(int, l.split(","))) for l in buf.value.decode().split()]
    wts, st, gl = gastar.parse_grid(doc)
    o, _ = oracle.grid_astar(wts, st, gl, path=False)
    assert oracle.grid_validate(wts, st, gl, [y * 6 + x for x, y in cells]) == (True, o.cost)


def test_cli_end_to_end(gastar, oracle, tmp_path):
    s, g = gastar.gen_sliding(3, 7400, 60, 60)
    f = tmp_path / "in.txt"
    f.write_text(f"{gastar.format_sliding(s)} {gastar.format_sliding(g)}\n")
    p = subprocess.run([CLI, "--version", "sliding", "--input-data", str(f)], capture_output=True,
                       text=True, check=True)
    lines = p.stdout.split()
    int(lines[0])  # milliseconds
    path = np.array([[0 if t == "_" else int(t) for t in l.split(",")] for l in lines[1:]], np.uint8)
    o, _ = oracle.sliding_astar(3, s, g, path=False)
    assert oracle.sliding_validate(3, s, g, path) == (True, o.cost)
    wts = gastar.gen_grid(60, 40, 7401, 0.2)
    obs = [(x, y) for y in range(40) for x in range(60) if wts[y, x] == 0]
    costs = [(x, y, int(wts[y, x])) for y in range(40) for x in range(60) if wts[y, x] > 1]
    doc = "60,40 0,0 59,39 %d %s %d %s\n" % (len(obs), " ".join(f"{x},{y}" for x, y in obs),
                                             len(costs), " ".join(f"{x},{y},{c}" for x, y, c in costs))
    out = tmp_path / "out.txt"
    subprocess.run([CLI, "--version", "pathfinding", "--output-data", str(out), "--delta", "18"],
                   input=doc, text=True, check=True)
    lines = out.read_text().split()
    cells = [tuple(map(int, l.split(","))) for l in lines[1:]]
    o, _ = oracle.grid_astar(wts, (0, 0), (59, 39), path=False)
    assert oracle.grid_validate(wts, (0, 0), (59, 39), [y * 60 + x for x, y in cells]) == (True, o.cost)
    # The same grid from the binary dense format.
    binf, out2 = tmp_path / "g.bin", tmp_path / "out2.txt"
    binf.write_bytes(gastar.encode_grid_binary(wts, (0, 0), (59, 39)))
    subprocess.run([CLI, "--version", "pathfinding", "--input-format", "binary", "--input-data", str(binf),
                    "--output-data", str(out2), "--delta", "18"], check=True)
    cells2 = [tuple(map(int, l.split(","))) for l in out2.read_text().split()[1:]]
    assert oracle.grid_validate(wts, (0, 0), (59, 39), [y * 60 + x for x, y in cells2]) == (True, o.cost)
