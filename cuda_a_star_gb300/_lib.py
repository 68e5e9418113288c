"""ctypes binding of libgastar.so (the C ABI declared in include/gastar.h).

The library is built in-tree (``cuda_a_star_gb300/_build/libgastar.so``).
Loading fails loudly when it is missing: there is no CPU fallback for the
search path.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgastar.so")

# Every symbol include/gastar.h declares (checked by the CPU test suite).
EXPORTS = [
    "gastar_config_default", "gastar_create", "gastar_destroy", "gastar_last_error",
    "gastar_status_name", "gastar_version", "gastar_device_info",
    "gastar_solve_sliding", "gastar_solve_grid", "gastar_solve_grid_device",
    "gastar_solve_sliding_noalloc", "gastar_grid_min_weight",
    "gastar_batch_config_default", "gastar_batch_create", "gastar_batch_destroy",
    "gastar_batch_add_sliding", "gastar_batch_add_grid", "gastar_batch_run",
    "gastar_batch_rerun", "gastar_batch_count", "gastar_batch_result", "gastar_batch_path",
    "gastar_batch_stats", "gastar_batch_autotune", "gastar_batch_phases", "gastar_batch_timeline",
    "gastar_serve_config_default", "gastar_serve_create", "gastar_serve_destroy",
    "gastar_serve_submit_sliding", "gastar_serve_submit_grid", "gastar_serve_step",
    "gastar_serve_poll", "gastar_serve_release", "gastar_serve_stats",
    "gastar_parse_sliding", "gastar_format_sliding", "gastar_parse_grid_dims",
    "gastar_parse_grid", "gastar_gen_sliding", "gastar_gen_grid",
    "gastar_format_grid", "gastar_encode_grid_binary", "gastar_decode_grid_header",
    "gastar_decode_grid_binary", "gastar_measure_random_peak", "gastar_measure_random_peak_ex",
]


class Config(C.Structure):
    _fields_ = [
        ("num_queues", C.c_uint32), ("heuristic", C.c_uint32), ("moves", C.c_uint32),
        ("expansion_width", C.c_uint32), ("warps_per_block", C.c_uint32),
        ("max_blocks", C.c_uint32), ("load_factor", C.c_float), ("table_log2", C.c_uint32),
        ("heap_entries", C.c_uint64), ("max_expansions", C.c_uint64),
        ("max_iterations", C.c_uint32), ("timeout_ms", C.c_uint32), ("regrow", C.c_uint32),
        ("delta", C.c_uint32), ("open_list", C.c_uint32), ("stream", C.c_void_p),
    ]


class Result(C.Structure):
    _fields_ = [
        ("status", C.c_int32), ("cost", C.c_uint32), ("path_len", C.c_uint32),
        ("iterations", C.c_uint32), ("expansions", C.c_uint64), ("generated", C.c_uint64),
        ("pushes", C.c_uint64), ("stale", C.c_uint64), ("table_used", C.c_uint64),
        ("kernel_ms", C.c_float), ("total_ms", C.c_float), ("attempts", C.c_uint32),
        ("launches", C.c_uint32), ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64),
    ]


class BatchConfig(C.Structure):
    _fields_ = [
        ("warps_per_block", C.c_uint32), ("expansion_width", C.c_uint32),
        ("load_factor", C.c_float), ("heuristic", C.c_uint32), ("moves", C.c_uint32),
        ("use_graph", C.c_uint32), ("blocks", C.c_uint32), ("timeout_ms", C.c_uint32),
        ("max_expansions", C.c_uint64), ("sliding_states", C.c_uint64),
        ("delta_grid", C.c_uint32), ("heavy_team", C.c_uint32), ("heavy_cells", C.c_uint64),
        ("promote_expansions", C.c_uint64), ("open_list", C.c_uint32), ("pad", C.c_uint32),
    ]


class ServeConfig(C.Structure):
    _fields_ = [
        ("budget_bytes", C.c_uint64), ("max_active", C.c_uint32), ("slice_iters", C.c_uint32),
        ("warps_per_block", C.c_uint32), ("expansion_width", C.c_uint32),
        ("load_factor", C.c_float), ("heuristic", C.c_uint32), ("moves", C.c_uint32),
        ("delta_grid", C.c_uint32), ("sliding_states", C.c_uint64),
        ("heavy_team", C.c_uint32), ("heavy_teams", C.c_uint32), ("heavy_cells", C.c_uint64),
        ("open_list", C.c_uint32), ("promote_log2", C.c_uint32),
        ("admit_bypass", C.c_uint32), ("weights_pool", C.c_uint32),
        ("weighted_slices", C.c_uint32), ("heavy_set", C.c_uint32),
    ]


_lib = None


def load(path: str | None = None) -> C.CDLL:
    """Loads libgastar.so (building it first only when asked by the caller)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"libgastar.so not found at {p}: build it with `python -m cuda_a_star_gb300.build` "
            "(the GA* engine has no CPU fallback)")
    lib = C.CDLL(p)
    u8p, u32p, vp = C.POINTER(C.c_uint8), C.POINTER(C.c_uint32), C.c_void_p
    sig = {
        "gastar_config_default": (None, [C.POINTER(Config)]),
        "gastar_create": (vp, [C.c_int]),
        "gastar_destroy": (None, [vp]),
        "gastar_last_error": (C.c_char_p, []),
        "gastar_status_name": (C.c_char_p, [C.c_int]),
        "gastar_version": (C.c_int, []),
        "gastar_device_info": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_uint64),
                                         C.c_char_p, C.c_size_t]),
        "gastar_solve_sliding": (C.c_int, [vp, C.c_uint32, u8p, u8p, C.POINTER(Config), u8p,
                                           C.c_uint32, C.POINTER(Result)]),
        "gastar_solve_sliding_noalloc": (C.c_int, [C.c_uint32, u8p, u8p, C.POINTER(Config), u8p,
                                                   C.c_uint32, C.POINTER(Result)]),
        "gastar_solve_grid": (C.c_int, [vp, C.c_uint32, C.c_uint32, u8p, C.c_uint32, C.c_uint32,
                                        C.c_uint32, C.c_uint32, C.POINTER(Config), u32p,
                                        C.c_uint32, C.POINTER(Result)]),
        "gastar_solve_grid_device": (C.c_int, [vp, C.c_uint32, C.c_uint32, vp, C.c_uint32,
                                               C.c_uint32, C.c_uint32, C.c_uint32,
                                               C.POINTER(Config), u32p, C.c_uint32,
                                               C.POINTER(Result)]),
        "gastar_grid_min_weight": (C.c_int, [vp, C.c_uint32, C.c_uint32, u8p, u32p, C.POINTER(C.c_int)]),
        "gastar_batch_config_default": (None, [C.POINTER(BatchConfig)]),
        "gastar_batch_create": (vp, [vp, C.POINTER(BatchConfig)]),
        "gastar_batch_destroy": (None, [vp]),
        "gastar_batch_add_sliding": (C.c_int, [vp, C.c_uint32, u8p, u8p]),
        "gastar_batch_add_grid": (C.c_int, [vp, C.c_uint32, C.c_uint32, u8p, C.c_uint32,
                                            C.c_uint32, C.c_uint32, C.c_uint32]),
        "gastar_batch_run": (C.c_int, [vp]),
        "gastar_batch_rerun": (C.c_int, [vp]),
        "gastar_batch_count": (C.c_uint32, [vp]),
        "gastar_batch_result": (C.c_int, [vp, C.c_uint32, C.POINTER(Result)]),
        "gastar_batch_path": (C.c_int, [vp, C.c_uint32, vp, C.c_uint32, u32p]),
        "gastar_batch_stats": (C.c_int, [vp, C.POINTER(C.c_float), C.POINTER(C.c_uint64),
                                         C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
        "gastar_batch_phases": (C.c_int, [vp, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                          C.POINTER(C.c_float), u32p, u32p]),
        "gastar_batch_timeline": (C.c_int, [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
        "gastar_batch_autotune": (C.c_int, [vp, C.c_uint32, C.c_char_p, C.POINTER(BatchConfig),
                                            C.POINTER(C.c_float)]),
        "gastar_serve_config_default": (None, [C.POINTER(ServeConfig)]),
        "gastar_serve_create": (vp, [vp, C.POINTER(ServeConfig)]),
        "gastar_serve_destroy": (None, [vp]),
        "gastar_serve_submit_sliding": (C.c_int64, [vp, C.c_uint32, u8p, u8p]),
        "gastar_serve_submit_grid": (C.c_int64, [vp, C.c_uint32, C.c_uint32, u8p, C.c_uint32,
                                                 C.c_uint32, C.c_uint32, C.c_uint32]),
        "gastar_serve_step": (C.c_int, [vp]),
        "gastar_serve_poll": (C.c_int, [vp, C.c_int64, C.POINTER(Result), vp, C.c_uint32, u32p]),
        "gastar_serve_release": (C.c_int, [vp, C.c_int64]),
        "gastar_serve_stats": (C.c_int, [vp, u32p, u32p, C.POINTER(C.c_uint64),
                                         C.POINTER(C.c_uint64), C.POINTER(C.c_float)]),
        "gastar_parse_sliding": (C.c_int, [C.c_char_p, C.c_uint32, u8p, u8p]),
        "gastar_format_sliding": (C.c_int, [C.c_uint32, u8p, C.c_char_p, C.c_size_t]),
        "gastar_parse_grid_dims": (C.c_int, [C.c_char_p, u32p, u32p]),
        "gastar_parse_grid": (C.c_int, [C.c_char_p, C.c_uint32, C.c_uint32, u8p, u32p, u32p,
                                        u32p, u32p]),
        "gastar_gen_sliding": (C.c_int, [C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32, u8p,
                                         u8p]),
        "gastar_gen_grid": (C.c_int, [C.c_uint32, C.c_uint32, C.c_uint64, C.c_double,
                                      C.c_uint32, C.c_uint32, u8p]),
        "gastar_format_grid": (C.c_int, [C.c_uint32, C.c_uint32, u8p, C.c_uint32, C.c_uint32,
                                         C.c_uint32, C.c_uint32, C.c_char_p, C.c_size_t,
                                         C.POINTER(C.c_size_t)]),
        "gastar_encode_grid_binary": (C.c_int, [C.c_uint32, C.c_uint32, u8p, C.c_uint32,
                                                C.c_uint32, C.c_uint32, C.c_uint32, u8p,
                                                C.c_size_t, C.POINTER(C.c_size_t)]),
        "gastar_decode_grid_header": (C.c_int, [u8p, C.c_size_t, u32p, u32p]),
        "gastar_measure_random_peak": (C.c_int, [vp, C.c_uint64, C.c_uint32,
                                                 C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "gastar_measure_random_peak_ex": (C.c_int, [vp, C.c_uint64, C.c_uint32, C.c_uint32,
                                                    C.c_uint32, C.POINTER(C.c_double),
                                                    C.POINTER(C.c_double)]),
        "gastar_decode_grid_binary": (C.c_int, [u8p, C.c_size_t, u8p, C.c_size_t, u32p, u32p,
                                                u32p, u32p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib
