"""Benchmark of the GA* search path on one GB300.

Default workload (the plain GA* configuration the metric is quoted on):
64 15-puzzles, each scrambled from the goal by a seeded non-reversing random
walk of uniform length 40-80, solved one instance per launch with 16384
parallel pops per iteration and a 2^30-slot duplicate-detection table.  A
step solves all 64 instances (search + path rebuild).

Output: one JSON line (rank 0).  `value` = solves/s with the instances
resident on the device (CUDA events on the launching stream); `e2e` = the same
through the C ABI with host buffers, copies included; `cpu_baseline` = the
single-thread host A* (the CPU oracle) over all host cores on the same
instances.  Beside the headline (rank 0, one GPU):
  p8          -- the single 8-puzzle instance, per-solve latency;
  grid_4096   -- plain GA* on the 4096 x 4096 weighted grid;
  batched     -- 1024 mixed instances in one persistent launch vs the plain
                 engine on a sample, its own roofline and e2e, every cost
                 checked against the oracle, paths validated on a sample;
  served      -- 512 mixed requests under Poisson arrivals at three loads,
                 p50/p99 overall and per class, every cost checked against
                 the oracle, the plain engine on a sample of the same mix;
  reference_gpu -- the reference's own CUDA GA* beside the engine on grids
                 in the reference's range (child process).
`--impl reference` times the CPU implementation (the oracle's A*) as the
reference arm: the reference itself has no CPU path.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = {
    "name": "P15 plain GA*: 64 x 15-puzzle (random walk 40-80 from goal 0..15), one instance "
            "per launch, Q=16384 parallel pops, 2^30-slot table",
    "n": 4, "instances": 64, "walk": (40, 80), "seed0": 0x15_0000, "num_queues": 16384,
    "table_log2": 30,
}


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    return rank, world


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def _config() -> dict:
    """The `config` of the headline workload, identical in both arms."""
    return {"workload": WORKLOAD["name"], "instances": WORKLOAD["instances"],
            "num_queues": WORKLOAD["num_queues"], "table_slots": 1 << WORKLOAD["table_log2"],
            "l2": "512 MiB buffer written between timed steps; 16 GiB table"}


def gen_sliding_host(n: int, seed: int, walk_min: int, walk_max: int):
    """The seeded scramble of gastar_gen_sliding, in plain Python (so that the
    CPU reference arm does not load the engine library): SplitMix64 (Steele,
    Lea, Flood 2014) draws the walk length and the moves of the blank from
    the goal 0..n*n-1, rejecting off-board moves and immediate reversals."""
    import numpy as np
    mask = (1 << 64) - 1
    state = seed & mask

    def nxt():
        nonlocal state
        state = (state + 0x9E3779B97F4A7C15) & mask
        z = state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
        return z ^ (z >> 31)

    def below(k):
        return ((nxt() >> 32) * k) >> 32

    goal = np.arange(n * n, dtype=np.uint8)
    start = goal.copy()
    length = walk_min + below(walk_max - walk_min + 1)
    dr, dc = (1, -1, 0, 0), (0, 0, 1, -1)
    blank, last, done = 0, -1, 0
    while done < length:
        m = below(4)
        if last >= 0 and m == (last ^ 1):
            continue
        row, col = blank // n + dr[m], blank % n + dc[m]
        if not (0 <= row < n and 0 <= col < n):
            continue
        q = row * n + col
        start[blank], start[q] = start[q], 0
        blank, last, done = q, m, done + 1
    return start, goal


def _instances(g=None, rank: int = 0):
    """The workload's instances; replica rank r gets its own seeds.  With the
    engine package `g` they come from its generator, else from the same
    generator in plain Python."""
    n = WORKLOAD["n"]
    lo, hi = WORKLOAD["walk"]
    base = WORKLOAD["seed0"] + rank * 1_000_000
    gen = g.gen_sliding if g is not None else gen_sliding_host
    return [gen(n, base + i, lo, hi) for i in range(WORKLOAD["instances"])]


def _cpu_model() -> str:
    """Host CPU model (lscpu's model name, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith(("model name", "cpu model")):
                    return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def _job_ms(local_ms: float, world: int) -> float:
    """The job's timed duration: the maximum over the ranks' timed regions."""
    if world == 1:
        return local_ms
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([local_ms], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _job_value(units_per_rank: int, steps: int, world: int, job_ms: float) -> float:
    """Whole-job throughput: the units all ranks processed / the job's time."""
    return units_per_rank * steps * world / (job_ms / 1000.0)


def _oracle_run(insts, threads=0):
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import numpy as np
    import oracle_lib as o
    starts = np.stack([s for s, _ in insts])
    goals = np.stack([g for _, g in insts])
    t0 = time.perf_counter()
    used, res = o.sliding_batch(WORKLOAD["n"], starts, goals, heuristic=o.ADM, threads=threads)
    dt = time.perf_counter() - t0
    return used, res, dt


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.p = None
        self.device = device
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(device), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
            out, _ = self.p.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


MIXED = {
    "name": "Batched GA*: 1024 mixed instances in one persistent launch -- 512 15-puzzles "
            "(random walk 20-80) + 512 weighted grids (side 256-2048, weights 1-9, obstacle "
            "density 0.1-0.3, corridor-guaranteed path)",
    "p15": 512, "grids": 512, "walk": (20, 80), "side": (256, 2048), "density": (0.1, 0.3),
    "seed0": 0x3_0000,
}


def _mixed_instances(g):
    import numpy as np
    rng = np.random.default_rng(MIXED["seed0"])
    p15 = [g.gen_sliding(4, MIXED["seed0"] + i, *MIXED["walk"]) for i in range(MIXED["p15"])]
    grids = []
    for i in range(MIXED["grids"]):
        side = int(rng.integers(MIXED["side"][0], MIXED["side"][1] + 1))
        dens = float(rng.uniform(*MIXED["density"]))
        grids.append((g.gen_grid(side, side, MIXED["seed0"] + 100_000 + i, dens), side))
    return p15, grids


# Pop window of the plain engine's grid solves (one grid over the whole GPU,
# bound by iteration latency): wider windows mean fewer iterations; on the
# 4096^2 and 8192^2 grids the time falls up to 54 and is flat from 54 to 144.
GRID_DELTA_PLAIN = 72


def run_grid4k(g, eng, check: bool) -> dict:
    """Plain GA* on the 4096 x 4096 weighted grid (weights 1..9, 20 %
    obstacles, monotone corridor (0,0) -> (4095,4095)): device time of the
    solve, expansions/s, and its cost against the CPU oracle."""
    wts = g.gen_grid(4096, 4096, 0x4096, 0.2)
    cfg = g.make_config(num_queues=16384, delta=GRID_DELTA_PLAIN)
    eng.solve_grid(wts, (0, 0), (4095, 4095), config=cfg)  # warm-up
    runs = [eng.solve_grid(wts, (0, 0), (4095, 4095), config=cfg) for _ in range(3)]
    r = min(runs, key=lambda x: x.kernel_ms)
    out = {"workload": "plain GA*, 4096x4096 grid, weights 1-9, 20% obstacles, corridor; Q=16384, "
                       f"pop window {GRID_DELTA_PLAIN}",
           "kernel_ms": r.kernel_ms, "total_ms": r.total_ms, "cost": r.cost,
           "node_expansions_per_s": r.expansions / (r.kernel_ms / 1000.0)}
    if check:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle_lib as o
        ref, _ = o.grid_astar(wts, (0, 0), (4095, 4095), path=False)
        out["oracle_cost"] = ref.cost
        out["optimal_cost_agreement"] = float(ref.cost == r.cost)
    return out


P8 = {"name": "Plain GA*: one 8-puzzle (goal 0..8 row-major, blank at 0; scrambled by a "
                "seeded random walk of 60 non-reversing blank moves), one instance per launch",
      "seed": 0x8_0060, "walk": 60}


def run_p8(g, eng, steps: int, check: bool) -> dict:
    """The single 8-puzzle instance of the plain configuration: per-solve latency
    through the C ABI (host buffers, path copied back) and its kernel time."""
    s, goal = g.gen_sliding(3, P8["seed"], P8["walk"], P8["walk"])
    for _ in range(3):
        eng.solve_sliding(s, goal, 3, path=True)
    reps = max(50, 10 * steps)
    rs = [eng.solve_sliding(s, goal, 3, path=True) for _ in range(reps)]
    tot = [r.total_ms for r in rs]
    out = {"workload": P8["name"], "solves": reps, "cost": rs[0].cost,
           "solves_per_s": reps / (sum(tot) / 1000.0),
           "e2e_ms": {"p50": _pct(tot, 0.5), "p99": _pct(tot, 0.99)},
           "kernel_ms": {"p50": _pct([r.kernel_ms for r in rs], 0.5)},
           "expansions": rs[0].expansions, "launches_per_solve": rs[0].launches,
           "how": "gastar_solve_sliding with host boards, path copied back; host wall time "
                  "per call (the instance is one launch: latency is the metric)"}
    if check:
        o = _oracle_lib()
        ref, _ = o.sliding_astar(3, s, goal, path=False)
        out["oracle_cost"] = ref.cost
        out["optimal_cost_agreement"] = sum(r.cost == ref.cost for r in rs) / reps
    return out


def reference_gpu_case() -> dict:
    """The reference's own GA* (oracle/_ref/libref_gpu.so, built from its
    unmodified headers) beside the engine's plain solve on inputs in the
    reference's range: grids up to 255 per side whose cells cost 2..9 (where its
    Manhattan heuristic is consistent, so both return the optimum).  Runs in a
    child process of the bench."""
    import ctypes as C
    import cuda_a_star_gb300 as g
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build as oracle_build
    try:
        path = oracle_build.build_ref_gpu()
    except Exception as exc:  # reported, never silently dropped
        return {"unavailable": f"build failed: {exc}"}
    if path is None:
        return {"unavailable": "reference headers not staged in oracle/_ref/src"}
    lib = C.CDLL(path)
    lib.ref_gpu_solve.argtypes = [C.c_int, C.c_int, C.c_char_p, C.c_uint32, C.c_char_p, C.c_size_t,
                                  C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.ref_gpu_error.restype = C.c_char_p
    rows = []
    with g.Engine(0) as eng:
        for i, (w, h) in enumerate([(64, 64), (128, 128), (200, 150), (255, 255)]):
            wts = g.gen_grid(w, h, 0x4EF0 + i, 0.2, wmin=2)
            text = g.format_grid(wts, (0, 0), (w - 1, h - 1)).encode()
            out = C.create_string_buffer(1 << 22)
            sm, wm = C.c_double(), C.c_double()
            ln = lib.ref_gpu_solve(1, 0, text, 4096, out, 1 << 22, C.byref(sm), C.byref(wm))
            if ln < 0:
                return {"unavailable": "reference solve failed: " + lib.ref_gpu_error().decode()}
            pts = [tuple(int(v) for v in t.split(",")) for t in out.value.decode().split()]
            ref_cost = int(sum(int(wts[y, x]) for x, y in pts[1:]))
            eng.solve_grid(wts, (0, 0), (w - 1, h - 1), num_queues=4096)
            e = [eng.solve_grid(wts, (0, 0), (w - 1, h - 1), num_queues=4096) for _ in range(5)]
            rows.append({"grid": f"{w}x{h}", "reference_search_ms": sm.value,
                         "reference_solve_ms": wm.value, "engine_solve_ms": min(x.total_ms for x in e),
                         "reference_cost": ref_cost, "engine_cost": e[0].cost})
    sp = sorted(r["reference_search_ms"] / r["engine_solve_ms"] for r in rows)
    return {"what": "reference's own CUDA GA* (a_star.h, Q=4096) vs this engine's plain solve "
                    "(Q=4096), same grids; reference search-loop time (its own clock) and whole "
                    "solve; engine wall time per call incl. copies and path",
            "grids": rows, "costs_equal": all(r["reference_cost"] == r["engine_cost"] for r in rows),
            "median_speedup_vs_reference_search": sp[len(sp) // 2]}


def _reference_gpu_subprocess() -> dict:
    try:
        p = subprocess.run([sys.executable, os.path.abspath(__file__), "--reference-gpu-case"],
                           capture_output=True, text=True, timeout=600)
    except subprocess.TimeoutExpired:
        return {"unavailable": "reference run exceeded 600 s"}
    for ln in reversed(p.stdout.splitlines()):
        if ln.startswith("{"):
            return json.loads(ln)
    return {"unavailable": f"reference run exited {p.returncode}: {p.stderr.strip()[-300:]}"}


def _oracle_lib():
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as o
    return o


def _check_batched(g, p15, grids, res) -> dict:
    """Optimal-cost agreement of every batched result with the CPU oracle
    (single-thread A* per instance over all host threads), and move-by-move
    path validity on a sample of 64 instances per class."""
    import numpy as np
    o = _oracle_lib()
    t0 = time.perf_counter()
    _, ref_p = o.sliding_batch(4, np.stack([s for s, _ in p15]), np.stack([t for _, t in p15]),
                               heuristic=o.ADM, threads=0)
    # largest grids first: the batch runner hands instances out in order
    order = sorted(range(len(grids)), key=lambda i: -grids[i][1])
    _, ref_g = o.grid_batch([(grids[i][0], (0, 0), (grids[i][1] - 1, grids[i][1] - 1)) for i in order],
                            heuristic=o.ADM, threads=0)
    ref = [r.cost if r.status == o.OK else None for r in ref_p]
    by_grid = [None] * len(grids)
    for k, i in enumerate(order):
        by_grid[i] = ref_g[k].cost if ref_g[k].status == o.OK else None
    ref += by_grid
    agree = sum(1 for r, c in zip(res, ref) if r.status == g.OK and r.cost == c)
    valid = {"p15": 0, "grid": 0}
    step = max(1, len(p15) // 64)
    for i in range(0, len(p15), step):
        r = res[i]
        valid["p15"] += r.path is not None and o.sliding_validate(4, *p15[i], r.path) == (True, r.cost)
    step = max(1, len(grids) // 64)
    for j in range(0, len(grids), step):
        r, (w, side) = res[len(p15) + j], grids[j]
        valid["grid"] += r.path is not None and o.grid_validate(
            w, (0, 0), (side - 1, side - 1), r.path) == (True, r.cost)
    return {"optimal_cost_agreement": agree / len(res), "agreeing": agree,
            "checked": len(res), "paths_valid": valid,
            "paths_checked": {"p15": len(range(0, len(p15), max(1, len(p15) // 64))),
                              "grid": len(range(0, len(grids), max(1, len(grids) // 64)))},
            "oracle_s": time.perf_counter() - t0}


def _traffic_ratio(name: str):
    """ncu's DRAM bytes / algorithmic bytes for a kernel on a small case of the
    workload (profiles/<name>.json), or None."""
    prof = os.path.join(ROOT, "profiles", name)
    if os.path.exists(prof):
        with open(prof) as f:
            return json.load(f).get("traffic_over_algorithmic")
    return None


def run_batched(g, eng, steps: int, check: bool = True) -> dict:
    """Batched mixed workload: one persistent launch over 1024 instances (autotuned),
    against the plain engine on a stratified 64-instance sample of the mix."""
    p15, grids = _mixed_instances(g)

    def fill(b):
        for s, goal in p15:
            b.add_sliding(s, goal)
        for w, side in grids:
            b.add_grid(w, (0, 0), (side - 1, side - 1))

    tuner = eng.batch()
    fill(tuner)
    build_dir = os.path.join(ROOT, "cuda_a_star_gb300", "_build")
    cache = os.path.join(build_dir, "autotune_cache.txt") if os.path.isdir(build_dir) else None
    t0 = time.perf_counter()
    tuned = tuner.autotune(sample=128, cache_path=cache)
    tune_s = time.perf_counter() - t0
    tuner.close()
    cfgkw = {k: tuned[k] for k in ("warps_per_block", "expansion_width", "load_factor",
                                    "delta_grid", "heavy_team", "heavy_cells", "open_list")}
    # end to end: host buffers -> upload -> solve -> results and paths back;
    # the median of three runs (one run is exposed to host-side noise)
    e2e_runs, e2e_kernel_ms = [], []
    for rep in range(3):
        if rep:
            b.close()
        t0 = time.perf_counter()
        b = eng.batch(**cfgkw)
        fill(b)
        b.run()
        res_paths = [b.result(i, path=True) for i in range(len(b))]
        e2e_runs.append(time.perf_counter() - t0)
        e2e_kernel_ms.append(b.stats()["kernel_ms"])
    e2e_s = statistics.median(e2e_runs)
    st0 = b.stats()
    # device-resident reruns (graph replay)
    kms, phases = [], None
    for _ in range(steps):
        b.rerun()
        phases = b.stats()
        kms.append(phases["kernel_ms"])
    res = [b.result(i, path=False) for i in range(len(b))]
    n = len(res)
    ok = sum(1 for r in res if r.status == g.OK)
    exp = sum(r.expansions for r in res)
    alg = sum(16 * (r.expansions + r.stale) + 32 * r.generated + 48 * r.pushes for r in res)
    ms = statistics.median(kms)
    lat = sorted(r.kernel_ms for r in res)
    b.close()
    # plain engine, one instance per launch, on a stratified sample of the mix
    sample = list(range(0, len(p15), 16)) + [len(p15) + i for i in range(0, len(grids), 16)]
    t_plain = 0.0
    for i in sample:
        if i < len(p15):
            r = eng.solve_sliding(*p15[i], 4, num_queues=16384, path=True, path_cap=1024)
        else:
            w, side = grids[i - len(p15)]
            r = eng.solve_grid(w, (0, 0), (side - 1, side - 1), num_queues=16384, delta=GRID_DELTA_PLAIN,
                               path=True)
        t_plain += r.total_ms / 1000.0
    plain_sps = len(sample) / t_plain
    peak, peak_kind = _peaks()
    main_ms = phases["main_ms"] if phases else ms
    # the persistent launch's algorithmic bytes over its own time: the re-solves
    # of overflowed instances run afterwards on the plain engine
    achieved = alg / (ms / 1000.0) / 1e9
    ratio = _traffic_ratio("search_kernel_batched.json")
    out = {
        "workload": MIXED["name"], "instances": n, "solved": ok,
        "solves_per_s": n / (ms / 1000.0), "node_expansions_per_s": exp / (ms / 1000.0),
        "ms_per_step": ms,
        "e2e": {"value": n / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": st0["h2d_bytes"],
                "d2h_bytes_per_step": st0["d2h_bytes"],
                "runs_s": [round(x, 4) for x in e2e_runs],
                "runs_kernel_ms": [round(x, 1) for x in e2e_kernel_ms],
                "how": "gastar_batch_create/add/run/result with host buffers, paths copied back; "
                       "median of 3"},
        "device_bytes": st0["device_bytes"],
        "instance_device_ms": {"p50": lat[n // 2], "p99": lat[min(n - 1, int(n * 0.99))],
                               "max": lat[-1]},
        "autotuned": cfgkw, "autotune_s": tune_s,
        "last_step_phases_ms": {k: phases[k] for k in ("main_ms", "retry_ms", "promote_ms",
                                                       "retried", "promoted")} if phases else None,
        "roofline": {"bound": "hbm", "kernel": "search_kernel (persistent batch launch) + plain "
                                               "re-solves of overflowed instances",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind,
                     "traffic": ratio * alg if ratio else None,
                     "traffic_source": "ncu DRAM bytes / algorithmic bytes on the batched profile "
                                       "case x this step's algorithmic bytes" if ratio else None,
                     "algorithmic_bytes": "16 B per pop + 32 B per generated successor "
                                          "+ 48 B per pushed successor"},
        "main_launch_ms": main_ms,
        "plain_same_mix_solves_per_s": plain_sps,
        "plain_sample": f"{len(sample)} instances (every 16th of each class), one per launch",
        "batched_over_plain": (n / (ms / 1000.0)) / plain_sps,
    }
    if check:
        out["oracle_check"] = _check_batched(g, p15, grids, res_paths)
        # the device-resident reruns solve the same instances: their costs too
        out["oracle_check"]["rerun_costs_equal_first_run"] = all(
            a.cost == b_.cost and a.status == b_.status for a, b_ in zip(res, res_paths))
    return out


SERVED = {
    "name": "Served GA*: Poisson arrivals of mixed requests -- 8-puzzles (walk 60), 15-puzzles "
            "(walk 20-80), 24-puzzles (walk 20-40), weighted grids (side 512-8192, weights 1-9, "
            "20% obstacles); 120 GiB device budget for request partitions",
    "requests": 512, "loads": (0.5, 0.9, 1.2), "seed0": 0x5_0000,
}
SERVED_CLASSES = ("p8", "p15", "p24", "grid")  # request i has class i % 4


def _served_requests(g):
    import numpy as np
    rng = np.random.default_rng(SERVED["seed0"])
    reqs = []
    for i in range(SERVED["requests"]):
        k = i % 4
        seed = SERVED["seed0"] + i
        if k == 0:
            reqs.append(("s", *g.gen_sliding(3, seed, 60, 60)))
        elif k == 1:
            reqs.append(("s", *g.gen_sliding(4, seed, 20, 80)))
        elif k == 2:
            reqs.append(("s", *g.gen_sliding(5, seed, 20, 40)))
        else:
            side = int(rng.integers(512, 8193))
            w = g.gen_grid(side, side, seed, 0.2)
            reqs.append(("g", w, (0, 0), (side - 1, side - 1)))
    return reqs


def _served_oracle(reqs):
    """Optimal cost of every request from the CPU oracle (all host threads)."""
    import numpy as np
    o = _oracle_lib()
    t0 = time.perf_counter()
    costs = [None] * len(reqs)
    for n, cls in ((3, 0), (4, 1), (5, 2)):
        idx = [i for i in range(len(reqs)) if i % 4 == cls]
        _, rr = o.sliding_batch(n, np.stack([reqs[i][1] for i in idx]),
                                np.stack([reqs[i][2] for i in idx]), heuristic=o.ADM, threads=0)
        for i, r in zip(idx, rr):
            costs[i] = r.cost if r.status == o.OK else None
    idx = sorted((i for i in range(len(reqs)) if i % 4 == 3), key=lambda i: -reqs[i][1].size)
    _, rr = o.grid_batch([(reqs[i][1], reqs[i][2], reqs[i][3]) for i in idx], heuristic=o.ADM,
                         threads=0)
    for i, r in zip(idx, rr):
        costs[i] = r.cost if r.status == o.OK else None
    return costs, time.perf_counter() - t0


def _pct(v, q):
    v = sorted(v)
    return v[min(len(v) - 1, int(len(v) * q))] if v else None


def run_served(g, eng, check: bool = True) -> dict:
    """Served mixed workload: the continuous-batching server under Poisson arrivals at
    three offered loads, calibrated to its capacity on a burst of the mix; every
    result checked against the oracle; the plain engine on a sample of the same mix."""
    import numpy as np
    reqs = _served_requests(g)
    srv = eng.server(budget_bytes=120 << 30)

    def submit(r):
        return srv.submit_sliding(r[1], r[2]) if r[0] == "s" else srv.submit_grid(r[1], r[2], r[3])

    def run(arrivals, paths=False):
        k0 = srv.stats()["kernel_ms"]
        t0 = time.perf_counter()
        ids, res, nxt = {}, {}, 0
        order = np.argsort(arrivals, kind="stable")
        pending = set()
        t_submit = 0.0
        while len(res) < len(reqs):
            now = time.perf_counter() - t0
            while nxt < len(order) and arrivals[order[nxt]] <= now:
                ts = time.perf_counter()
                i = submit(reqs[order[nxt]])
                t_submit += time.perf_counter() - ts
                ids[i] = int(order[nxt])
                pending.add(i)
                nxt += 1
            st = srv.stats()
            if st["active"] or st["waiting"]:
                srv.step()
            elif nxt < len(order):
                time.sleep(max(0.0, min(0.002, arrivals[order[nxt]] - now)))
            for i in list(pending):
                r = srv.poll(i, path=paths)
                if r is not None:
                    res[ids[i]] = r
                    pending.discard(i)
        wall = time.perf_counter() - t0
        kernel_s = (srv.stats()["kernel_ms"] - k0) / 1000.0
        for i in ids:
            srv.release(i)
        lat = [res[k].total_ms for k in range(len(reqs))]
        out = {"solves_per_s": len(reqs) / wall, "wall_s": wall,
               "submit_s": t_submit, "search_kernel_s": kernel_s,
               "node_expansions_per_s": sum(r.expansions for r in res.values()) / wall,
               "latency_ms": {"p50": _pct(lat, 0.5), "p99": _pct(lat, 0.99)},
               "latency_ms_by_class": {
                   c: {"p50": _pct(lat[k::4], 0.5), "p99": _pct(lat[k::4], 0.99),
                       "max": max(lat[k::4])} for k, c in enumerate(SERVED_CLASSES)},
               "expansions_by_class": {c: sum(res[j].expansions for j in range(k, len(reqs), 4))
                                       for k, c in enumerate(SERVED_CLASSES)},
               "algorithmic_bytes": sum(16 * (r.expansions + r.stale) + 32 * r.generated
                                        + 48 * r.pushes for r in res.values()),
               "solved": sum(1 for r in res.values() if r.status == g.OK)}
        return out, res

    burst, burst_res = run(np.zeros(len(reqs)), paths=check)
    cap = burst["solves_per_s"]
    rng = np.random.default_rng(SERVED["seed0"] + 1)
    loads, load_res = {}, {}
    for f in SERVED["loads"]:
        rate = f * cap
        arrivals = np.cumsum(rng.exponential(1.0 / rate, size=len(reqs)))
        out, res = run(arrivals)
        out["offered_per_s"] = rate
        loads[f"{f}x"] = out
        load_res[f"{f}x"] = res
    srv.close()
    # plain engine, one request per launch, on every 4th request of each class
    sample = [i for i in range(len(reqs)) if (i // 4) % 4 == 0]
    t_plain = 0.0
    for i in sample:
        r = reqs[i]
        if r[0] == "s":
            x = eng.solve_sliding(r[1], r[2], path=True, path_cap=1024)
        else:
            x = eng.solve_grid(r[1], r[2], r[3], num_queues=16384, delta=GRID_DELTA_PLAIN, path=True)
        t_plain += x.total_ms / 1000.0
    plain_sps = len(sample) / t_plain
    out = {"workload": SERVED["name"], "requests": len(reqs), "capacity_solves_per_s": cap,
           "burst": burst, "loads": loads,
           "plain_same_mix_solves_per_s": plain_sps,
           "plain_sample": f"{len(sample)} requests (every 4th of each class), one per launch, "
                           f"paths included",
           "served_over_plain": cap / plain_sps}
    if check:
        costs, osec = _served_oracle(reqs)

        def agree(res):
            return sum(1 for k, r in res.items() if r.status == g.OK and r.cost == costs[k]) / len(reqs)

        o = _oracle_lib()
        valid, checked = {c: 0 for c in SERVED_CLASSES}, {c: 0 for c in SERVED_CLASSES}
        for k in range(len(reqs)):
            if (k // 4) % 2:
                continue  # 64 per class
            c, r, q = SERVED_CLASSES[k % 4], burst_res[k], reqs[k]
            checked[c] += 1
            if r.path is None:
                continue
            if q[0] == "s":
                n = int(round(len(q[1]) ** 0.5))
                valid[c] += o.sliding_validate(n, q[1], q[2], r.path) == (True, r.cost)
            else:
                valid[c] += o.grid_validate(q[1], q[2], q[3], r.path) == (True, r.cost)
        out["burst"]["optimal_cost_agreement"] = agree(burst_res)
        for f, res in load_res.items():
            out["loads"][f]["optimal_cost_agreement"] = agree(res)
        out["oracle_check"] = {"paths_valid": valid, "paths_checked": checked, "oracle_s": osec}
    return out


def run_reference(args) -> dict:
    """The CPU implementation of the path (host A*, all host threads).  The
    reference has no CPU path of its own; this arm runs the oracle's
    single-thread A* per instance, one instance per host thread, on the same
    64 instances (generated here without the engine library)."""
    insts = _instances()
    for _ in range(args.warmup):
        _oracle_run(insts)
    times, used = [], 0
    for _ in range(args.steps):
        used, res, dt = _oracle_run(insts)
        times.append(dt)
    total = sum(times)
    value = WORKLOAD["instances"] * args.steps / total
    return {
        "impl": "reference", "metric": "solves/s", "value": value, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": _config(),
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": used, "kind": "port",
                         "cpu_model": _cpu_model(),
                         "sample": f"all {WORKLOAD['instances']} instances per step, "
                                   f"single-thread A* per instance over {used} host threads"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "expansions_per_s": sum(r.expansions for r in res) / times[-1],
    }


def run_ours(args) -> dict:
    import numpy as np
    import torch
    import cuda_a_star_gb300 as g
    from cuda_a_star_gb300 import build as engine_build

    engine_build.build()
    rank, world = _dist()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    eng = g.Engine(dev)
    stream = torch.cuda.current_stream()
    cfg = g.make_config(num_queues=WORKLOAD["num_queues"], table_log2=WORKLOAD["table_log2"],
                        stream=stream.cuda_stream)
    insts = _instances(g, rank)  # replicas: every rank its own 64 instances
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    def step(collect):
        out = []
        for s, goal in insts:
            r = eng.solve_sliding(s, goal, WORKLOAD["n"], config=cfg, path=True, path_cap=1024)
            if r.status != g.OK:
                raise RuntimeError(f"solve failed: {r.status_name}")
            if collect:
                out.append(r)
        return out

    for _ in range(max(args.warmup, 0)):
        step(False)
    # --- device-timed steps (inputs resident; L2 flushed between steps) ---
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(dev)
    step_ms, results = [], []
    for k in range(args.steps):
        flush.fill_(k & 0xff)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        rs = step(True)
        e1.record(stream)
        torch.cuda.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        results.extend(rs)
    clk = clocks.stop()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    # --- end-to-end steps through the C ABI with host buffers ---
    e2e_s, h2d, d2h = [], 0, 0
    for k in range(args.steps):
        flush.fill_((k + 7) & 0xff)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rs = step(True)
        torch.cuda.synchronize()
        e2e_s.append(time.perf_counter() - t0)
        h2d = sum(r.h2d_bytes for r in rs)
        d2h = sum(r.d2h_bytes for r in rs)
    total_ms = _job_ms(sum(step_ms), world)
    n_inst = WORKLOAD["instances"]
    value = _job_value(n_inst, args.steps, world, total_ms)
    exp = sum(r.expansions for r in results)
    lat = sorted(r.total_ms for r in results)
    kern_s = sum(r.kernel_ms for r in results) / 1000.0
    alg_bytes = sum(16 * (r.expansions + r.stale) + 32 * r.generated + 48 * r.pushes for r in results)
    launches = sum(r.launches for r in results)
    peak, peak_kind = _peaks()
    achieved = alg_bytes / kern_s / 1e9 if kern_s > 0 else 0.0
    # DRAM traffic per launch: ncu's traffic/algorithmic ratio of the same
    # kernel on instances of this workload, applied to this run's launches.
    traffic = None
    prof = os.path.join(ROOT, "profiles", "search_kernel_p15.json")
    searches = len(results)
    if os.path.exists(prof) and searches:
        with open(prof) as f:
            ratio = json.load(f).get("traffic_over_algorithmic")
        if ratio:
            traffic = ratio * alg_bytes / searches
    out = {
        "metric": "solves/s", "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic",
        "config": _config(),
        "node_expansions_per_s": exp / (total_ms / 1000.0),
        "latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[min(len(lat) - 1, int(len(lat) * 0.99))]},
        "e2e": {"value": n_inst * args.steps / sum(e2e_s), "unit": "solves/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                     "kernel": "search_kernel",
                     "algorithmic_bytes": "16 B per pop + 32 B per generated successor "
                                          "+ 48 B per pushed successor"},
        "clocks": clk,
    }
    # The search's memory traffic is random 16-32 byte accesses (table slots,
    # heap nodes): its own roofline is the device's measured random-sector
    # rate, reported beside the streaming-copy fraction above.
    try:
        # The device's random-sector rate at the table's size (16 GiB), swept
        # over accesses in flight and loads per sector; the maximum is the
        # denominator (the full sweep: bench.py --random-sweep).
        rows = eng.random_access_sweep(kinds=("gather", "cas"), buffers=(16 << 30,),
                                       in_flight=(8, 16, 32), loads_per_sector=(1, 2))
        rg = max((r for r in rows if r["kind"] == "gather"), key=lambda r: r["gbs"])
        rc = max((r for r in rows if r["kind"] == "cas"), key=lambda r: r["gbs"])
        out["roofline"]["random_access"] = {
            "gather_gbs": rg["gbs"], "cas16_gbs": rc["gbs"], "unit": "GB/s",
            "frac_of_gather": achieved / rg["gbs"] if rg["gbs"] > 0 else None,
            "gather_best_shape": {k: rg[k] for k in ("buffer_bytes", "in_flight", "loads_per_sector")},
            "how": "random 32-byte sector loads / random 16-byte CAS over a 16 GiB buffer (the "
                   "table's size), max over 8/16/32 accesses in flight per thread and 1/2 loads "
                   "per sector; sectors x 32 B / kernel time (gastar_measure_random_peak_ex)"}
    except Exception as exc:  # reported, never silently dropped
        out["roofline"]["random_access"] = {"error": str(exc)}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        used, res, dt = _oracle_run(insts)
        costs_gpu = [r.cost for r in results[:n_inst]]
        agree = sum(1 for a, b in zip(costs_gpu, res) if a == b.cost) / n_inst
        per = sorted(1000.0 * r.seconds for r in res)
        out["cpu_baseline"] = {"value": n_inst / dt, "unit": "solves/s", "cores": used,
                               "kind": "port", "cpu_model": _cpu_model(),
                               "sample": f"the same {n_inst} instances once, single-thread host "
                                         f"A* per instance over {used} threads",
                               "per_instance_ms_one_core": {
                                   "p50": per[len(per) // 2], "mean": sum(per) / len(per),
                                   "max": per[-1],
                                   "how": "each instance's own time on the core that solved it "
                                          f"({used} instances running at once)"}}
        out["optimal_cost_agreement"] = agree
    if rank == 0 and world == 1:
        out["p8"] = run_p8(g, eng, args.steps, check=not args.no_cpu_baseline)
        out["grid_4096"] = run_grid4k(g, eng, check=not args.no_cpu_baseline)
    if rank == 0 and world == 1 and not args.no_batched:
        out["batched"] = run_batched(g, eng, max(1, min(args.steps, 3)),
                                     check=not args.no_cpu_baseline)
        ra = out["roofline"].get("random_access", {})
        if ra.get("gather_gbs"):
            out["batched"]["roofline"]["frac_of_random_gather"] = (
                out["batched"]["roofline"]["achieved"] / ra["gather_gbs"])
    if rank == 0 and world == 1 and not args.no_served:
        out["served"] = run_served(g, eng, check=not args.no_cpu_baseline)
        bu = out["served"]["burst"]
        if bu.get("search_kernel_s"):
            ach = bu["algorithmic_bytes"] / bu["search_kernel_s"] / 1e9
            peak, peak_kind = out["roofline"]["peak"], out["roofline"]["peak_source"]
            bu["roofline"] = {"bound": "hbm", "kernel": "search_kernel (served slices; plain "
                                                        "re-solves of promoted puzzles included)",
                              "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                              "peak_source": peak_kind,
                              "algorithmic_bytes": "16 B per pop + 32 B per generated successor "
                                                   "+ 48 B per pushed successor, summed over "
                                                   "the burst's 512 results / search-kernel time"}
            ra = out["roofline"].get("random_access", {})
            if ra.get("gather_gbs"):
                bu["roofline"]["frac_of_random_gather"] = ach / ra["gather_gbs"]
    if world > 1:
        torch.distributed.destroy_process_group()
    eng.close()
    if rank == 0 and world == 1 and not args.no_reference_gpu:
        out["reference_gpu"] = _reference_gpu_subprocess()
    return out if rank == 0 else {}


def run_profile_case(kind: str) -> None:
    """Small copies of the workloads for ncu captures (a few GB on the device).
    plain: 4 of the 64 P15 instances, 2^24-slot table, one launch each.
    batched: 32 P15 (walk 20-80) + 32 grids (side 256-512), a run and a re-run.
    grid: the 4096^2 grid solved twice (upload kernel, search, path rebuild).
    served: two 4096^2 grids on eight-block teams in a server (2 GiB budget)."""
    import cuda_a_star_gb300 as g
    from cuda_a_star_gb300 import build as engine_build
    engine_build.build()

    def alg(r):  # algorithmic bytes of one solve
        return 16 * (r.expansions + r.stale) + 32 * r.generated + 48 * r.pushes

    with g.Engine(0) as eng:
        if kind == "plain":
            cfg = g.make_config(num_queues=WORKLOAD["num_queues"], table_log2=24)
            for s, goal in _instances(g)[:4]:
                r = eng.solve_sliding(s, goal, WORKLOAD["n"], config=cfg, path=True, path_cap=1024)
                print(json.dumps({"status": r.status_name, "cost": r.cost, "expansions": r.expansions,
                                  "generated": r.generated, "pushes": r.pushes, "stale": r.stale,
                                  "iterations": r.iterations, "kernel_ms": r.kernel_ms,
                                  "algorithmic_bytes": alg(r)}))
            return
        if kind == "served":
            srv = eng.server(budget_bytes=2 << 30)
            reqs = [g.gen_grid(4096, 4096, 0x5E00 + i, 0.2) for i in range(2)]
            ids = [srv.submit_grid(w, (0, 0), (4095, 4095)) for w in reqs]
            out = srv.drain(ids)
            for i in ids:
                r = out[i]
                print(json.dumps({"status": r.status_name, "cost": r.cost, "expansions": r.expansions,
                                  "generated": r.generated, "pushes": r.pushes, "stale": r.stale,
                                  "iterations": r.iterations, "algorithmic_bytes": alg(r)}))
            print(json.dumps({"search_kernel_ms": srv.stats()["kernel_ms"]}))
            srv.close()
            return
        if kind == "grid":
            wts = g.gen_grid(4096, 4096, 0x4096, 0.2)
            for _ in range(2):
                r = eng.solve_grid(wts, (0, 0), (4095, 4095), num_queues=16384, delta=GRID_DELTA_PLAIN,
                                   path=True)
                print(json.dumps({"status": r.status_name, "cost": r.cost, "path_len": len(r.path),
                                  "kernel_ms": r.kernel_ms, "total_ms": r.total_ms,
                                  "upload_path": eng.grid_min_weight(wts[:16, :16])[1]}))
            return
        p15, grids = _mixed_instances(g)
        b = eng.batch(warps_per_block=16, expansion_width=32, load_factor=0.5, delta_grid=18)
        for s, goal in p15[:32]:
            b.add_sliding(s, goal)
        small = [(w, side) for w, side in grids if side <= 512][:32]
        for w, side in small:
            b.add_grid(w, (0, 0), (side - 1, side - 1))
        # First run (fresh partitions: whole tables cleared), then a
        # device-resident re-run (only the slots the first run claimed are
        # cleared): the batch kernel's second launch is the re-run's.
        for label in ("run", "rerun"):
            b.run() if label == "run" else b.rerun()
            res = [b.result(i, path=False) for i in range(len(b))]
            print(json.dumps({"launch": label, "instances": len(res),
                              "solved": sum(r.status == g.OK for r in res),
                              "expansions": sum(r.expansions for r in res),
                              "algorithmic_bytes": sum(alg(r) for r in res),
                              "stats": b.stats()}))
        b.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched mixed workload")
    ap.add_argument("--no-served", action="store_true", help="skip the served workload")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="skip the reference's own CUDA GA* beside the engine on small grids")
    ap.add_argument("--reference-gpu-case", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--profile-case", nargs="?", const="plain", choices=["plain", "batched", "grid", "served"],
                    help="small single pass for ncu captures (no bench JSON line)")
    ap.add_argument("--random-sweep", action="store_true",
                    help="print the random-access rate over buffer size, depth in flight and "
                         "loads per sector (JSON), no bench line")
    args = ap.parse_args()
    if args.random_sweep:
        import cuda_a_star_gb300 as g
        from cuda_a_star_gb300 import build as engine_build
        engine_build.build()
        with g.Engine(0) as eng:
            for row in eng.random_access_sweep():
                print(json.dumps(row))
        return
    if args.reference_gpu_case:
        print(json.dumps(reference_gpu_case()))
        return
    if args.profile_case:
        run_profile_case(args.profile_case)
        return
    rank, world = _dist()
    if args.impl == "reference":
        if rank != 0:
            return
        out = run_reference(args)
    else:
        out = run_ours(args)
    if rank == 0 and out:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
