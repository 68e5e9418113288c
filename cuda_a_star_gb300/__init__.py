"""Python host API of the GB300 GA* engine (libgastar.so over its C ABI).

Mirrors the reference's front ends (michalborkowski96/cuda_a_star):
``SlidingPuzzle::solve<size>`` (a_star_sliding_puzzle.h:165-171) and
``Pathfinding::solve`` (a_star_pathfinding.h:223-238) become
:meth:`Engine.solve_sliding` / :meth:`Engine.solve_grid`, and
:func:`solve_sliding_text` / :func:`solve_grid_text` read the reference's text
input and return ``(path, milliseconds)`` like the reference's ``solve``.
Errors come back as :class:`GastarError` (the reference throws
``std::runtime_error``, helpers.h:46-50).
"""
from __future__ import annotations

import ctypes as C
import weakref
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import BatchConfig, Config, Result, ServeConfig  # noqa: F401  (re-exported)

H_ADMISSIBLE, H_REFERENCE, H_ZERO = 0, 1, 2
MOVES_STANDARD, MOVES_REFERENCE = 0, 1

STATUS = ["OK", "NO_PATH", "BUDGET", "TIMEOUT", "HEAP_FULL", "TABLE_FULL", "PATH_CAP",
          "BARRIER_TIMEOUT", "BAD_INPUT", "CUDA_ERROR", "NO_DEVICE", "PENDING", "OUT_OF_MEMORY",
          "COST_RANGE"]
OK, NO_PATH = 0, 1


class GastarError(RuntimeError):
    pass


def _u8p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_uint8))


def _u32p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def lib():
    return _lib.load()


def _check(rc: int, what: str) -> None:
    if rc != 0:
        msg = lib().gastar_last_error().decode()
        name = STATUS[rc] if 0 <= rc < len(STATUS) else str(rc)
        raise GastarError(f"{what}: {name} {msg}")


@dataclass
class SolveResult:
    status: int
    cost: int
    path: np.ndarray | None
    expansions: int = 0
    generated: int = 0
    pushes: int = 0
    stale: int = 0
    iterations: int = 0
    table_used: int = 0
    kernel_ms: float = 0.0
    total_ms: float = 0.0
    attempts: int = 1
    launches: int = 0
    h2d_bytes: int = 0
    d2h_bytes: int = 0
    extra: dict = field(default_factory=dict)

    @property
    def status_name(self) -> str:
        return STATUS[self.status] if 0 <= self.status < len(STATUS) else str(self.status)

    @staticmethod
    def from_c(r: Result, path) -> "SolveResult":
        return SolveResult(r.status, r.cost, path, r.expansions, r.generated, r.pushes, r.stale,
                           r.iterations, r.table_used, r.kernel_ms, r.total_ms, r.attempts,
                           r.launches, r.h2d_bytes, r.d2h_bytes)


def make_config(num_queues: int = 4096, heuristic: int = H_ADMISSIBLE,
                moves: int = MOVES_STANDARD, **kw) -> Config:
    cfg = Config()
    lib().gastar_config_default(C.byref(cfg))
    cfg.num_queues = num_queues
    cfg.heuristic = heuristic
    cfg.moves = moves
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


class Engine:
    """One GPU context (device memory, stream, events) reused across solves."""

    def __init__(self, device: int = 0):
        self._h = lib().gastar_create(device)
        if not self._h:
            raise GastarError("gastar_create: " + lib().gastar_last_error().decode())
        self._batches: "weakref.WeakSet[Batch]" = weakref.WeakSet()

    def close(self) -> None:
        # Batches borrow the context: release them first.
        for b in list(self._batches):
            b.close()
        if self._h:
            lib().gastar_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def device_info(self) -> dict:
        sms, mem = C.c_int(), C.c_uint64()
        name = C.create_string_buffer(256)
        lib().gastar_device_info(self._h, C.byref(sms), C.byref(mem), name, 256)
        return {"sms": sms.value, "mem_bytes": mem.value, "name": name.value.decode()}

    def solve_sliding(self, start, goal, n: int | None = None, config: Config | None = None,
                      path: bool = True, path_cap: int = 4096, **kw) -> SolveResult:
        s = np.ascontiguousarray(start, dtype=np.uint8).reshape(-1)
        g = np.ascontiguousarray(goal, dtype=np.uint8).reshape(-1)
        n = n or int(round(len(s) ** 0.5))
        cfg = config or make_config(**kw)
        res = Result()
        buf = np.zeros((path_cap, n * n), dtype=np.uint8) if path else None
        rc = lib().gastar_solve_sliding(self._h, n, _u8p(s), _u8p(g), C.byref(cfg),
                                        _u8p(buf) if path else None, path_cap if path else 0,
                                        C.byref(res))
        _check(rc, "gastar_solve_sliding")
        p = buf[:res.path_len].copy() if (path and res.status == OK) else None
        return SolveResult.from_c(res, p)

    def solve_grid(self, weights, start, goal, config: Config | None = None, path: bool = True,
                   **kw) -> SolveResult:
        w8 = np.ascontiguousarray(weights, dtype=np.uint8)
        h, w = w8.shape
        cfg = config or make_config(**kw)
        res = Result()
        cap = w * h if path else 0
        buf = np.zeros(max(cap, 1), dtype=np.uint32)
        rc = lib().gastar_solve_grid(self._h, w, h, _u8p(w8), start[0], start[1], goal[0], goal[1],
                                     C.byref(cfg), _u32p(buf) if path else None, cap, C.byref(res))
        _check(rc, "gastar_solve_grid")
        p = buf[:res.path_len].copy() if (path and res.status == OK) else None
        return SolveResult.from_c(res, p)

    def solve_grid_device(self, d_weights_ptr: int, w: int, h: int, start, goal,
                          config: Config | None = None, **kw) -> SolveResult:
        cfg = config or make_config(**kw)
        res = Result()
        rc = lib().gastar_solve_grid_device(self._h, w, h, C.c_void_p(d_weights_ptr), start[0],
                                            start[1], goal[0], goal[1], C.byref(cfg), None, 0,
                                            C.byref(res))
        _check(rc, "gastar_solve_grid_device")
        return SolveResult.from_c(res, None)

    UPLOAD_PATHS = ("copy", "inplace", "staged")

    def grid_min_weight(self, weights) -> tuple[int, str]:
        """Least passable weight of a grid as the engine computes it (255: none),
        and the upload path that brought the weights to the device."""
        w8 = np.ascontiguousarray(weights, dtype=np.uint8)
        h, w = w8.shape
        mw, up = C.c_uint32(), C.c_int()
        _check(lib().gastar_grid_min_weight(self._h, w, h, _u8p(w8), C.byref(mw), C.byref(up)),
               "gastar_grid_min_weight")
        return mw.value, self.UPLOAD_PATHS[up.value]

    def random_access_peak(self, kind: str = "gather", buffer_bytes: int = 8 << 30) -> dict:
        """Measured random 32-byte-sector rate (GB/s): "gather" loads or "cas"
        16-byte compare-and-swaps, the roofline of the table and heap kernels."""
        gbs, ms = C.c_double(), C.c_double()
        _check(lib().gastar_measure_random_peak(self._h, buffer_bytes, 0 if kind == "gather" else 1,
                                                C.byref(gbs), C.byref(ms)), "random_access_peak")
        return {"kind": kind, "gbs": gbs.value, "ms": ms.value}

    def random_access_sweep(self, kinds=("gather", "cas"),
                            buffers=(64 << 20, 256 << 20, 1 << 30, 4 << 30, 16 << 30),
                            in_flight=(2, 4, 8, 16, 32), loads_per_sector=(1, 2)) -> list[dict]:
        """The random 32-byte-sector rate over buffer size, accesses in flight
        per thread and (gather) 16-byte loads per sector: one row per point."""
        rows = []
        for kind in kinds:
            k = 0 if kind == "gather" else 1
            for b in buffers:
                for f in in_flight:
                    for lp in (loads_per_sector if k == 0 else (1,)):
                        gbs, ms = C.c_double(), C.c_double()
                        _check(lib().gastar_measure_random_peak_ex(self._h, b, k, f, lp, C.byref(gbs),
                                                                   C.byref(ms)), "random_access_sweep")
                        rows.append({"kind": kind, "buffer_bytes": b, "in_flight": f,
                                     "loads_per_sector": lp, "gbs": gbs.value, "ms": ms.value})
        return rows

    def batch(self, **kw) -> "Batch":
        return Batch(self, **kw)

    def server(self, **kw) -> "Server":
        return Server(self, **kw)


class Batch:
    """Many instances solved by one persistent launch (see gastar_batch_*)."""

    def __init__(self, engine: Engine, **kw):
        cfg = BatchConfig()
        lib().gastar_batch_config_default(C.byref(cfg))
        for k, v in kw.items():
            setattr(cfg, k, v)
        self.cfg = cfg
        self.engine = engine
        self._h = lib().gastar_batch_create(engine._h, C.byref(cfg))
        if not self._h:
            raise GastarError("gastar_batch_create failed")
        engine._batches.add(self)
        self.kinds: list[tuple] = []

    def close(self):
        if self._h:
            lib().gastar_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_sliding(self, start, goal) -> int:
        s = np.ascontiguousarray(start, dtype=np.uint8).reshape(-1)
        g = np.ascontiguousarray(goal, dtype=np.uint8).reshape(-1)
        n = int(round(len(s) ** 0.5))
        i = lib().gastar_batch_add_sliding(self._h, n, _u8p(s), _u8p(g))
        if i < 0:
            _check(-i, "gastar_batch_add_sliding")
        self.kinds.append(("sliding", n))
        return i

    def add_grid(self, weights, start, goal) -> int:
        w8 = np.ascontiguousarray(weights, dtype=np.uint8)
        h, w = w8.shape
        i = lib().gastar_batch_add_grid(self._h, w, h, _u8p(w8), start[0], start[1], goal[0], goal[1])
        if i < 0:
            _check(-i, "gastar_batch_add_grid")
        self.kinds.append(("grid", w * h))
        return i

    def autotune(self, sample: int = 64, cache_path: str | None = None) -> dict:
        """Picks the batch configuration for this instance mix (before run())."""
        out = BatchConfig()
        ms = C.c_float()
        _check(lib().gastar_batch_autotune(self._h, sample,
                                           cache_path.encode() if cache_path else None,
                                           C.byref(out), C.byref(ms)), "gastar_batch_autotune")
        self.cfg = out
        return {"warps_per_block": out.warps_per_block, "expansion_width": out.expansion_width,
                "load_factor": round(out.load_factor, 3), "delta_grid": out.delta_grid,
                "heavy_team": out.heavy_team, "heavy_cells": out.heavy_cells,
                "open_list": out.open_list, "trial_ms": ms.value}

    def run(self) -> None:
        _check(lib().gastar_batch_run(self._h), "gastar_batch_run")

    def rerun(self) -> None:
        _check(lib().gastar_batch_rerun(self._h), "gastar_batch_rerun")

    def __len__(self) -> int:
        return lib().gastar_batch_count(self._h)

    def result(self, i: int, path: bool = True) -> SolveResult:
        r = Result()
        _check(lib().gastar_batch_result(self._h, i, C.byref(r)), "gastar_batch_result")
        p = None
        if path and r.status == OK:
            kind, size = self.kinds[i]
            if kind == "grid":
                buf = np.zeros(r.path_len, dtype=np.uint32)
            else:
                buf = np.zeros((r.path_len, size * size), dtype=np.uint8)
            ln = C.c_uint32()
            _check(lib().gastar_batch_path(self._h, i, buf.ctypes.data_as(C.c_void_p), r.path_len,
                                           C.byref(ln)), "gastar_batch_path")
            p = buf
        return SolveResult.from_c(r, p)

    def timeline(self):
        """(start_ns, end_ns) arrays of the last run's persistent launch, one
        entry per instance, from the earliest start; 0, 0 where none ran."""
        import numpy as np
        n = len(self)
        s = np.zeros(n, dtype=np.uint64)
        e = np.zeros(n, dtype=np.uint64)
        _check(lib().gastar_batch_timeline(self._h, s.ctypes.data_as(C.POINTER(C.c_uint64)),
                                           e.ctypes.data_as(C.POINTER(C.c_uint64))),
               "gastar_batch_timeline")
        return s, e

    def stats(self) -> dict:
        ms, h2d, d2h, dev = C.c_float(), C.c_uint64(), C.c_uint64(), C.c_uint64()
        lib().gastar_batch_stats(self._h, C.byref(ms), C.byref(h2d), C.byref(d2h), C.byref(dev))
        a, r, p = C.c_float(), C.c_float(), C.c_float()
        nr, npr = C.c_uint32(), C.c_uint32()
        lib().gastar_batch_phases(self._h, C.byref(a), C.byref(r), C.byref(p), C.byref(nr),
                                  C.byref(npr))
        return {"kernel_ms": ms.value, "h2d_bytes": h2d.value, "d2h_bytes": d2h.value,
                "device_bytes": dev.value, "main_ms": a.value, "retry_ms": r.value,
                "promote_ms": p.value, "retried": nr.value, "promoted": npr.value}


class Server:
    """Continuous-batching request loop (see gastar_serve_*)."""

    PENDING = 11

    def __init__(self, engine: Engine, **kw):
        cfg = ServeConfig()
        lib().gastar_serve_config_default(C.byref(cfg))
        for k, v in kw.items():
            setattr(cfg, k, v)
        self.cfg = cfg
        self._h = lib().gastar_serve_create(engine._h, C.byref(cfg))
        if not self._h:
            raise GastarError("gastar_serve_create: " + lib().gastar_last_error().decode())
        engine._batches.add(self)
        self.kinds: dict[int, tuple] = {}

    def close(self):
        if self._h:
            lib().gastar_serve_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit_sliding(self, start, goal) -> int:
        s = np.ascontiguousarray(start, dtype=np.uint8).reshape(-1)
        g = np.ascontiguousarray(goal, dtype=np.uint8).reshape(-1)
        n = int(round(len(s) ** 0.5))
        i = lib().gastar_serve_submit_sliding(self._h, n, _u8p(s), _u8p(g))
        if i < 0:
            _check(-i, "gastar_serve_submit_sliding")
        self.kinds[i] = ("sliding", n)
        return i

    def submit_grid(self, weights, start, goal) -> int:
        w8 = np.ascontiguousarray(weights, dtype=np.uint8)
        h, w = w8.shape
        i = lib().gastar_serve_submit_grid(self._h, w, h, _u8p(w8), start[0], start[1], goal[0],
                                           goal[1])
        if i < 0:
            _check(-i, "gastar_serve_submit_grid")
        self.kinds[i] = ("grid", w * h)
        return i

    def step(self) -> None:
        _check(lib().gastar_serve_step(self._h), "gastar_serve_step")

    def poll(self, i: int, path: bool = True) -> SolveResult | None:
        r = Result()
        rc = lib().gastar_serve_poll(self._h, i, C.byref(r), None, 0, None)
        if rc == self.PENDING:
            return None
        _check(rc, "gastar_serve_poll")
        p = None
        if path and r.status == OK:
            kind, size = self.kinds[i]
            buf = (np.zeros(r.path_len, dtype=np.uint32) if kind == "grid"
                   else np.zeros((r.path_len, size * size), dtype=np.uint8))
            ln = C.c_uint32()
            _check(lib().gastar_serve_poll(self._h, i, C.byref(r), buf.ctypes.data_as(C.c_void_p),
                                           r.path_len, C.byref(ln)), "gastar_serve_poll")
            p = buf
        return SolveResult.from_c(r, p)

    def release(self, i: int) -> None:
        lib().gastar_serve_release(self._h, i)
        self.kinds.pop(i, None)

    def stats(self) -> dict:
        wt, ac = C.c_uint32(), C.c_uint32()
        done, used = C.c_uint64(), C.c_uint64()
        ms = C.c_float()
        lib().gastar_serve_stats(self._h, C.byref(wt), C.byref(ac), C.byref(done), C.byref(used),
                                 C.byref(ms))
        return {"waiting": wt.value, "active": ac.value, "completed": done.value,
                "bytes_in_use": used.value, "kernel_ms": ms.value}

    def drain(self, ids, max_steps: int = 1_000_000) -> dict:
        """Steps until every id in `ids` is finished; returns id -> SolveResult."""
        out = {}
        pending = set(ids)
        for _ in range(max_steps):
            if not pending:
                break
            self.step()
            for i in list(pending):
                r = self.poll(i)
                if r is not None:
                    out[i] = r
                    pending.discard(i)
        if pending:
            raise GastarError(f"{len(pending)} requests still pending")
        return out


# ---- host-only helpers (no GPU needed) ----

def gen_sliding(n: int, seed: int, walk_min: int, walk_max: int) -> tuple[np.ndarray, np.ndarray]:
    s = np.zeros(n * n, dtype=np.uint8)
    g = np.zeros(n * n, dtype=np.uint8)
    _check(lib().gastar_gen_sliding(n, seed, walk_min, walk_max, _u8p(s), _u8p(g)), "gen_sliding")
    return s, g


def gen_grid(w: int, h: int, seed: int, density: float = 0.2, wmin: int = 1,
             wmax: int = 9) -> np.ndarray:
    a = np.zeros((h, w), dtype=np.uint8)
    _check(lib().gastar_gen_grid(w, h, seed, density, wmin, wmax, _u8p(a)), "gen_grid")
    return a


def parse_sliding(text: str, n: int) -> tuple[np.ndarray, np.ndarray]:
    s = np.zeros(n * n, dtype=np.uint8)
    g = np.zeros(n * n, dtype=np.uint8)
    _check(lib().gastar_parse_sliding(text.encode(), n, _u8p(s), _u8p(g)), "parse_sliding")
    return s, g


def format_sliding(board) -> str:
    b = np.ascontiguousarray(board, dtype=np.uint8).reshape(-1)
    n = int(round(len(b) ** 0.5))
    buf = C.create_string_buffer(256)
    _check(lib().gastar_format_sliding(n, _u8p(b), buf, 256), "format_sliding")
    return buf.value.decode()


def parse_grid(text: str):
    w, h = C.c_uint32(), C.c_uint32()
    _check(lib().gastar_parse_grid_dims(text.encode(), C.byref(w), C.byref(h)), "parse_grid")
    a = np.zeros((h.value, w.value), dtype=np.uint8)
    sx, sy, tx, ty = (C.c_uint32() for _ in range(4))
    _check(lib().gastar_parse_grid(text.encode(), w.value, h.value, _u8p(a), C.byref(sx),
                                   C.byref(sy), C.byref(tx), C.byref(ty)), "parse_grid")
    return a, (sx.value, sy.value), (tx.value, ty.value)


def format_grid(weights, start, goal) -> str:
    """The reference's grid document (a_star_pathfinding.h:223-231, 83-128)."""
    a = np.ascontiguousarray(weights, dtype=np.uint8)
    h, w = a.shape
    need = C.c_size_t()
    lib().gastar_format_grid(w, h, _u8p(a), start[0], start[1], goal[0], goal[1], None, 0,
                             C.byref(need))
    buf = C.create_string_buffer(need.value)
    _check(lib().gastar_format_grid(w, h, _u8p(a), start[0], start[1], goal[0], goal[1], buf,
                                    need.value, C.byref(need)), "format_grid")
    return buf.value.decode()


def encode_grid_binary(weights, start, goal) -> bytes:
    """Binary dense grid: 32-byte header ("GAGRID1\\0", w, h, sx, sy, tx, ty as
    little-endian u32) then the w*h weights row-major."""
    a = np.ascontiguousarray(weights, dtype=np.uint8)
    h, w = a.shape
    out = np.zeros(32 + a.size, dtype=np.uint8)
    n = C.c_size_t()
    _check(lib().gastar_encode_grid_binary(w, h, _u8p(a), start[0], start[1], goal[0], goal[1],
                                           _u8p(out), out.size, C.byref(n)), "encode_grid_binary")
    return out[:n.value].tobytes()


def decode_grid_binary(data: bytes):
    buf = np.frombuffer(data, dtype=np.uint8).copy()
    w, h = C.c_uint32(), C.c_uint32()
    _check(lib().gastar_decode_grid_header(_u8p(buf), buf.size, C.byref(w), C.byref(h)),
           "decode_grid_binary")
    a = np.zeros((h.value, w.value), dtype=np.uint8)
    sx, sy, tx, ty = (C.c_uint32() for _ in range(4))
    _check(lib().gastar_decode_grid_binary(_u8p(buf), buf.size, _u8p(a), a.size, C.byref(sx),
                                           C.byref(sy), C.byref(tx), C.byref(ty)),
           "decode_grid_binary")
    return a, (sx.value, sy.value), (tx.value, ty.value)


def solve_sliding_text(engine: Engine, text: str, size: int, num_queues: int = 4096, **kw):
    """``SlidingPuzzle::solve<size>(in, num_queues)``: returns (boards, ms)."""
    s, g = parse_sliding(text, size)
    r = engine.solve_sliding(s, g, size, num_queues=num_queues, **kw)
    return (r.path if r.path is not None else np.zeros((0, size * size), np.uint8)), r.kernel_ms


def solve_grid_text(engine: Engine, text: str, num_queues: int = 4096, **kw):
    """``Pathfinding::solve(in, num_queues)``: returns ([(x, y), ...], ms)."""
    wts, st, gl = parse_grid(text)
    r = engine.solve_grid(wts, st, gl, num_queues=num_queues, **kw)
    w = wts.shape[1]
    path = [] if r.path is None else [(int(c % w), int(c // w)) for c in r.path]
    return path, r.kernel_ms
