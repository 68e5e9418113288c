/*
 * gastar — GA* (massively parallel A*) search engine for one NVIDIA GB300.
 * C ABI of libgastar.so.  Plain pointers and sizes only; every function
 * returns a status code instead of throwing.
 *
 * Each entry point names the reference interface (michalborkowski96/cuda_a_star)
 * it replaces.  Boards are n*n bytes row-major with 0 for the blank (the
 * reference's SlidingPuzzle::Position<size>::board, a_star_sliding_puzzle.h:14-18);
 * grids are w*h bytes indexed y*w + x holding the cost of entering the cell,
 * 0 for an impassable cell (the reference's obstacle and cost lists,
 * a_star_pathfinding.h:74-81, in dense form).
 */
#ifndef GASTAR_H
#define GASTAR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (per call and per solve) ---- */
enum gastar_status {
    GASTAR_OK = 0,             /* call succeeded / path found */
    GASTAR_NO_PATH = 1,        /* search space exhausted without reaching the goal */
    GASTAR_BUDGET = 2,         /* expansion or iteration budget exhausted */
    GASTAR_TIMEOUT = 3,        /* wall-clock deadline reached on the device */
    GASTAR_HEAP_FULL = 4,      /* a priority-queue partition ran out of nodes */
    GASTAR_TABLE_FULL = 5,     /* the duplicate-detection table passed its load limit */
    GASTAR_PATH_CAP = 6,       /* caller's path buffer too small (path_len holds the need) */
    GASTAR_BARRIER_TIMEOUT = 7,/* a device-side wait gave up (bounded spin) */
    GASTAR_BAD_INPUT = 8,      /* malformed instance or argument */
    GASTAR_CUDA_ERROR = 9,     /* CUDA runtime error (see gastar_last_error) */
    GASTAR_NO_DEVICE = 10,     /* no usable GPU */
    GASTAR_PENDING = 11,       /* serving: request not finished yet */
    GASTAR_OUT_OF_MEMORY = 12, /* device memory budget exceeded */
    GASTAR_COST_RANGE = 13,    /* a path cost reached 2^24 (the engine's cost range) */
};

enum gastar_heuristic {
    GASTAR_H_ADMISSIBLE = 0, /* tile Manhattan without the blank; Chebyshev x min weight on grids */
    GASTAR_H_REFERENCE = 1,  /* the reference's formulas: Manhattan incl. blank
                                (a_star_sliding_puzzle.h:152-163); Manhattan on grids
                                (a_star_pathfinding.h:219-221).  Not admissible. */
    GASTAR_H_ZERO = 2,       /* h = 0 (Dijkstra order) */
};

enum gastar_moves {
    GASTAR_MOVES_STANDARD = 0,  /* blank moves to any of its 4 neighbours */
    GASTAR_MOVES_REFERENCE = 1, /* the reference's successor arithmetic: only moves 0 (row+1)
                                   and 2 (col+1) exist (a_star_sliding_puzzle.h:106-111) */
};

/* Search parameters.  Zero fields take defaults (gastar_config_default). */
typedef struct gastar_config {
    uint32_t num_queues;       /* parallel pops per iteration (reference Q, main.cu:18) */
    uint32_t heuristic;        /* gastar_heuristic */
    uint32_t moves;            /* gastar_moves (sliding puzzles only) */
    uint32_t expansion_width;  /* entries each warp-heap pops per iteration, 1..32;
                                  0 = auto, clamp(num_queues / 1024, 8, 32), and a
                                  puzzle search on several blocks that passes 64
                                  iterations then pops twice as many (at most 32) */
    uint32_t warps_per_block;  /* warp-heaps per thread block, 1..16 (above 8: the
                                  512-thread kernel, at most 128 registers per thread);
                                  0 = auto (8 when the blocks still cover half of the
                                  SMs, else 4) */
    uint32_t max_blocks;       /* cap on thread blocks for one instance (0 = all SMs) */
    float load_factor;         /* table load limit before GASTAR_TABLE_FULL (0.5..0.9) */
    uint32_t table_log2;       /* hash-table slots = 2^table_log2 (0 = adaptive) */
    uint64_t heap_entries;     /* priority-queue capacity per instance (0 = adaptive) */
    uint64_t max_expansions;   /* 0 = unlimited */
    uint32_t max_iterations;   /* 0 = unlimited */
    uint32_t timeout_ms;       /* device-side deadline, 0 = none */
    uint32_t regrow;           /* plain engine: re-run with doubled capacity on *_FULL (default 1) */
    uint32_t delta;            /* pop window: expand only f <= min f + delta (0 = no window) */
    uint32_t open_list;        /* 0 = warp-heaps (top levels in shared memory);
                                  1 = shared-memory f-buckets in front of the warp-heaps */
    void *stream;              /* cudaStream_t to launch on (NULL = the context's stream) */
} gastar_config;

/* Outcome of one solve. */
typedef struct gastar_result {
    int32_t status;            /* gastar_status */
    uint32_t cost;             /* path cost (valid when status == GASTAR_OK) */
    uint32_t path_len;         /* states on the path, start and goal included */
    uint32_t iterations;       /* GA* iterations (pop/expand/push rounds) */
    uint64_t expansions;       /* non-stale pops that generated successors */
    uint64_t generated;        /* successors produced by the move function */
    uint64_t pushes;           /* successors that improved the table and were queued */
    uint64_t stale;            /* pops discarded because the table held a lower g */
    uint64_t table_used;       /* states stored in the duplicate-detection table */
    float kernel_ms;           /* device time of the search kernel(s), CUDA events; batch
                                  results: this instance's first-to-last iteration time */
    float total_ms;            /* host wall time of the call; batch results: whole launch;
                                  served results: submit -> completion */
    uint32_t attempts;         /* plain engine: solves run (1 + regrows) */
    uint32_t launches;         /* kernels this call launched */
    uint64_t h2d_bytes;        /* bytes copied host -> device by this call */
    uint64_t d2h_bytes;        /* bytes copied device -> host by this call */
} gastar_result;

typedef struct gastar_ctx gastar_ctx;

/* ---- context ---- */
void gastar_config_default(gastar_config *cfg);
/* Creates a context on `device` (-1 = current).  Returns NULL on failure. */
gastar_ctx *gastar_create(int device);
void gastar_destroy(gastar_ctx *ctx);
const char *gastar_last_error(void);
const char *gastar_status_name(int status);
int gastar_version(void);
/* Device properties the engine sized itself with: SM count, device memory. */
int gastar_device_info(gastar_ctx *ctx, int *sm_count, uint64_t *mem_bytes, char *name,
                       size_t name_len);

/* ---- plain GA*: one instance per launch ----
 * Replaces SlidingPuzzle::solve<size> + a_star<Position<size>, 4, ...>
 * (a_star_sliding_puzzle.h:165-171, a_star.h:223-282).  `path` receives up to
 * path_cap boards (n*n bytes each), start first.  path may be NULL. */
int gastar_solve_sliding(gastar_ctx *ctx, uint32_t n, const uint8_t *start, const uint8_t *goal,
                         const gastar_config *cfg, uint8_t *path, uint32_t path_cap,
                         gastar_result *out);
/* Replaces Pathfinding::solve + a_star<Position, 8, ...> (a_star_pathfinding.h:223-238).
 * `path` receives cell indices (y*w + x), start first. */
int gastar_solve_grid(gastar_ctx *ctx, uint32_t w, uint32_t h, const uint8_t *weights,
                      uint32_t sx, uint32_t sy, uint32_t tx, uint32_t ty,
                      const gastar_config *cfg, uint32_t *path, uint32_t path_cap,
                      gastar_result *out);
/* Device-resident variant of gastar_solve_grid: `d_weights` is a device
 * pointer; nothing is copied host->device.  path may be NULL. */
int gastar_solve_grid_device(gastar_ctx *ctx, uint32_t w, uint32_t h, const uint8_t *d_weights,
                             uint32_t sx, uint32_t sy, uint32_t tx, uint32_t ty,
                             const gastar_config *cfg, uint32_t *path, uint32_t path_cap,
                             gastar_result *out);

/* The least passable (non-zero) weight of a grid, 255 if none: the factor of
 * the admissible grid heuristic.  The weights reach the device as in
 * gastar_solve_grid, gastar_batch_add_grid and gastar_serve_submit_grid, by
 * the context's upload path (*upload_path; may be NULL): 2 = staged (default:
 * host threads copy into pinned chunks and reduce while earlier chunks are
 * sent), 1 = read in place by one kernel (GPUs that read pageable host
 * memory through the host's page tables, e.g. Grace systems), 0 = copied,
 * then reduced on the device.  The environment variable GASTAR_UPLOAD
 * (staged | inplace | copy) at gastar_create chooses.  No counterpart in the
 * reference (its grid heuristic takes no weight factor). */
int gastar_grid_min_weight(gastar_ctx *ctx, uint32_t w, uint32_t h, const uint8_t *weights,
                           uint32_t *minw, int *upload_path);

/* 8-puzzle solve that allocates nothing, for callers that cannot call
 * cudaMalloc (their device memory is reserved by another pool, or they must
 * avoid the device-wide synchronisation of cudaMalloc/cudaFree).  No
 * counterpart in the reference.  Arguments and result fields as
 * gastar_solve_sliding, without a context; n must be 3 (GASTAR_BAD_INPUT
 * otherwise).  Scratch is a fixed ~16 MiB device array inside the library,
 * held by every GPU that loads the library until exit; all calls share it, so
 * calls that overlap on the GPU race.  Every call looks up the array's address
 * on the current device, and synchronises the stream it runs on (cfg->stream,
 * or the legacy default stream when that is NULL) before it returns.
 * Fixed shape: one block of 4 warp-heaps popping 32 entries each, a 2^19-slot
 * table, 4095 nodes per warp-heap, a 4096-state path arena, no regrow; the
 * config fields num_queues, expansion_width, warps_per_block, max_blocks,
 * load_factor, table_log2, heap_entries, regrow and open_list are ignored
 * (heuristic, moves, max_expansions, max_iterations, timeout_ms, delta and
 * stream apply).  Costs equal gastar_solve_sliding's for the admissible and
 * zero heuristics (both optimal); with GASTAR_H_REFERENCE the cost depends on
 * the expansion order and may differ.  A path longer than the arena returns
 * GASTAR_PATH_CAP with the cost and path_len = cost + 1.  kernel_ms is 0. */
int gastar_solve_sliding_noalloc(uint32_t n, const uint8_t *start, const uint8_t *goal,
                                 const gastar_config *cfg, uint8_t *path, uint32_t path_cap,
                                 gastar_result *out);

/* ---- batched GA*: many instances in one persistent launch ----
 * No reference counterpart (the reference solves one instance per process,
 * its problem data lives in __constant__ symbols: a_star_sliding_puzzle.h:125-128,
 * a_star_pathfinding.h:72-81). */
typedef struct gastar_batch gastar_batch;
typedef struct gastar_batch_config {
    uint32_t warps_per_block;  /* warp-heaps per instance (queue count) */
    uint32_t expansion_width;  /* pops per warp-heap per iteration */
    float load_factor;         /* hash-table load factor used to size partitions */
    uint32_t heuristic, moves;
    uint32_t use_graph;        /* capture the launch sequence in a CUDA graph */
    uint32_t blocks;           /* persistent blocks (0 = occupancy x SMs) */
    uint32_t timeout_ms;
    uint64_t max_expansions;   /* per instance */
    uint64_t sliding_states;   /* expected max states per puzzle instance (0 = by size) */
    uint32_t delta_grid;       /* pop window for grid instances (0 = none) */
    uint32_t heavy_team;       /* blocks per team for heavy instances (1 = no teams) */
    uint64_t heavy_cells;      /* grids with at least this many cells are heavy */
    uint64_t promote_expansions; /* puzzles past this many expansions are re-solved by the
                                    plain engine on the whole GPU (0 = never) */
    uint32_t open_list;        /* 0 = warp-heaps; 1 (default) = f-buckets (pages in the
                                  partition) in front of the warp-heaps */
    uint32_t pad;
} gastar_batch_config;

void gastar_batch_config_default(gastar_batch_config *cfg);
gastar_batch *gastar_batch_create(gastar_ctx *ctx, const gastar_batch_config *cfg);
void gastar_batch_destroy(gastar_batch *b);
/* Returns the instance index (>= 0) or a negative gastar_status. */
int gastar_batch_add_sliding(gastar_batch *b, uint32_t n, const uint8_t *start,
                             const uint8_t *goal);
int gastar_batch_add_grid(gastar_batch *b, uint32_t w, uint32_t h, const uint8_t *weights,
                          uint32_t sx, uint32_t sy, uint32_t tx, uint32_t ty);
/* Allocates partitions, uploads instances (host->device) and solves them all. */
int gastar_batch_run(gastar_batch *b);
/* Re-solves the already uploaded instances (inputs resident in device memory). */
int gastar_batch_rerun(gastar_batch *b);
uint32_t gastar_batch_count(const gastar_batch *b);
int gastar_batch_result(gastar_batch *b, uint32_t index, gastar_result *out);
/* Copies the path of one solved instance: boards (sliding) or cell indices (grid). */
int gastar_batch_path(gastar_batch *b, uint32_t index, void *path, uint32_t path_cap,
                      uint32_t *path_len);
/* Autotuner: times trial batches over a stratified sample of `sample`
 * instances of this (not yet run) batch and keeps the fastest warp-heaps per
 * instance, expansion width, grid pop window, heavy-team size and table load
 * factor (coordinate descent).  The choice is applied to the batch, written
 * to `out` and cached per GPU and instance-mix signature in `cache_path`
 * (NULL = no cache); a cached signature skips the trials. */
int gastar_batch_autotune(gastar_batch *b, uint32_t sample, const char *cache_path,
                          gastar_batch_config *out, float *best_ms);
/* Device time of the last run's kernel(s) and the bytes copied each way. */
int gastar_batch_stats(gastar_batch *b, float *kernel_ms, uint64_t *h2d_bytes,
                       uint64_t *d2h_bytes, uint64_t *device_bytes);
/* Kernel time of the last run by phase: the persistent launch, the re-run of
 * overflowed instances with larger partitions, and the plain-engine re-solves
 * of promoted puzzles; with how many instances took the last two. */
int gastar_batch_phases(gastar_batch *b, float *main_ms, float *retry_ms, float *promote_ms,
                        uint32_t *retried, uint32_t *promoted);
/* Schedule of the last run's persistent launch: per instance (count entries),
 * the device times at which its search started and ended, in ns from the
 * earliest start; 0 and 0 for an instance that did not run (unreachable).
 * Re-runs and re-solves after the launch are not included. */
int gastar_batch_timeline(gastar_batch *b, uint64_t *start_ns, uint64_t *end_ns);

/* ---- served GA*: continuous batching of solve requests ----
 * No reference counterpart (one instance per process there).  Requests wait in
 * a FIFO queue; each gastar_serve_step admits waiting requests while a slot
 * and enough of the device-memory budget are free, runs one persistent launch
 * over every active request for at most slice_iters GA* iterations each (search
 * state stays resident between steps), rebuilds the paths of finished ones and
 * frees their memory.  total_ms of a polled result is submit -> completion. */
typedef struct gastar_server gastar_server;
typedef struct gastar_serve_config {
    uint64_t budget_bytes;     /* device bytes for request partitions (default 120 GiB) */
    uint32_t max_active;       /* requests on the device at once (0 = resident blocks) */
    uint32_t slice_iters;      /* iterations per request per step (default 128) */
    uint32_t warps_per_block;  /* warp-heaps per request */
    uint32_t expansion_width;  /* pops per warp-heap per iteration */
    float load_factor;
    uint32_t heuristic, moves;
    uint32_t delta_grid;       /* pop window for grid requests (0 = none) */
    uint64_t sliding_states;   /* expected max states per puzzle request (0 = by size) */
    uint32_t heavy_team;       /* blocks per team for heavy requests (1 = no teams) */
    uint32_t heavy_teams;      /* most teams per launch (0 = as many as the resident blocks
                                  hold); each launch leaves up to a quarter of the resident
                                  blocks to the one-block requests it has */
    uint64_t heavy_cells;      /* grids with at least this many cells are heavy */
    uint32_t open_list;        /* 0 = warp-heaps; 1 (default) = f-buckets (pages in the
                                  partition, state kept there between steps) in front of
                                  the warp-heaps */
    uint32_t promote_log2;     /* a 15- or 24-puzzle request past 2^promote_log2
                                  expansions leaves its slot and is finished by the plain
                                  engine on the whole GPU between two steps (0 = never;
                                  default 18) */
    uint32_t admit_bypass;     /* 1 (default) = a request needing at most 1/256 of the
                                  budget may be admitted ahead of a larger one waiting
                                  for memory; 0 = strict arrival order */
    uint32_t weights_pool;     /* 1 (default) = grid weights go from the caller's buffer
                                  to a device pool (an eighth of the budget, beside it)
                                  at submission; 0, or a full pool = a host copy, sent
                                  at admission */
    uint32_t weighted_slices;  /* 1 (default) = when only heavy requests are left, more of
                                  them than teams (the end of a burst), each gets
                                  1/2x..4x slice_iters in proportion to its estimated
                                  work left; 0 = equal */
    uint32_t heavy_set;        /* at most heavy_set x teams heavy requests, the largest
                                  first, take turns on the teams in a launch (default 4:
                                  fewer grids per launch keep their frontiers in L2);
                                  0 = all active ones */
} gastar_serve_config;

void gastar_serve_config_default(gastar_serve_config *cfg);
gastar_server *gastar_serve_create(gastar_ctx *ctx, const gastar_serve_config *cfg);
void gastar_serve_destroy(gastar_server *srv);
/* Returns a request id (>= 0) or a negative gastar_status. */
int64_t gastar_serve_submit_sliding(gastar_server *srv, uint32_t n, const uint8_t *start,
                                    const uint8_t *goal);
int64_t gastar_serve_submit_grid(gastar_server *srv, uint32_t w, uint32_t h,
                                 const uint8_t *weights, uint32_t sx, uint32_t sy, uint32_t tx,
                                 uint32_t ty);
/* One scheduling round: admit, one slice launch, retire finished requests. */
int gastar_serve_step(gastar_server *srv);
/* GASTAR_OK with the result (and path: boards or cell indices) when the
 * request is finished, GASTAR_PENDING otherwise. */
int gastar_serve_poll(gastar_server *srv, int64_t id, gastar_result *out, void *path,
                      uint32_t path_cap, uint32_t *path_len);
/* Forgets a finished request. */
int gastar_serve_release(gastar_server *srv, int64_t id);
int gastar_serve_stats(gastar_server *srv, uint32_t *waiting, uint32_t *active,
                       uint64_t *completed, uint64_t *bytes_in_use, float *kernel_ms);

/* Measured random-access peak of the device, the roofline denominator of the
 * table and heap kernels (no reference counterpart): kind 0 = random 32-byte
 * sector loads, kind 1 = random 16-byte compare-and-swaps, over a buffer of
 * the largest power of two <= buffer_bytes (at least 1 GiB, far above L2).
 * *gbs = sectors x 32 bytes / kernel time; *ms = that kernel time. */
int gastar_measure_random_peak(gastar_ctx *ctx, uint64_t buffer_bytes, uint32_t kind, double *gbs,
                               double *ms);
/* The same measurement with its shape as arguments, for sweeping the
 * denominator (no reference counterpart): the buffer is the largest power of
 * two <= buffer_bytes (at least 1 MiB, so L2-resident sizes are allowed);
 * in_flight = independent accesses each thread keeps outstanding (1, 2, 4, 8,
 * 16 or 32); loads_per_sector = 16-byte loads per 32-byte sector for kind 0
 * (1 or 2; either moves the whole sector).  GASTAR_BAD_INPUT otherwise. */
int gastar_measure_random_peak_ex(gastar_ctx *ctx, uint64_t buffer_bytes, uint32_t kind,
                                  uint32_t in_flight, uint32_t loads_per_sector, double *gbs,
                                  double *ms);

/* ---- text formats and synthetic instances (host only, no GPU needed) ---- */
/* Reads "start goal" in the reference's sliding format (Position(std::istream&),
 * a_star_sliding_puzzle.h:21-48): n*n comma-separated ints, "_" or "0" = blank. */
int gastar_parse_sliding(const char *text, uint32_t n, uint8_t *start, uint8_t *goal);
/* Prints a board like the reference's operator<< (a_star_sliding_puzzle.h:59-74). */
int gastar_format_sliding(uint32_t n, const uint8_t *board, char *out, size_t cap);
/* Reads the grid header "W,H" (a_star_pathfinding.h:224). */
int gastar_parse_grid_dims(const char *text, uint32_t *w, uint32_t *h);
/* Reads the full grid document (a_star_pathfinding.h:223-231, 83-128) into a
 * dense w*h weight array: unlisted cells cost 1, obstacles 0. */
int gastar_parse_grid(const char *text, uint32_t w, uint32_t h, uint8_t *weights, uint32_t *sx,
                      uint32_t *sy, uint32_t *tx, uint32_t *ty);
/* The reference's grid document for a dense weight array (obstacles = weight
 * 0, costs = weights other than 1); `*written` = bytes needed incl. the NUL. */
int gastar_format_grid(uint32_t w, uint32_t h, const uint8_t *weights, uint32_t sx, uint32_t sy,
                       uint32_t tx, uint32_t ty, char *out, size_t cap, size_t *written);
/* Binary dense grid: the 8 bytes "GAGRID1\0", then w, h, sx, sy, tx, ty as
 * little-endian u32, then the w*h weights row-major (0 = obstacle).  A 4096^2
 * grid is 16.8 MB instead of ~200 MB of reference text.  No reference
 * counterpart: it sits beside the text format (a_star_pathfinding.h:83-128). */
#define GASTAR_GRID_BINARY_HEADER 32
int gastar_encode_grid_binary(uint32_t w, uint32_t h, const uint8_t *weights, uint32_t sx, uint32_t sy,
                              uint32_t tx, uint32_t ty, uint8_t *out, size_t cap, size_t *written);
int gastar_decode_grid_header(const uint8_t *buf, size_t len, uint32_t *w, uint32_t *h);
int gastar_decode_grid_binary(const uint8_t *buf, size_t len, uint8_t *weights, size_t weights_cap,
                              uint32_t *sx, uint32_t *sy, uint32_t *tx, uint32_t *ty);
/* Seeded instances: goal 0..n*n-1 row-major, start = non-reversing random
 * walk of uniform length in [walk_min, walk_max] (SplitMix64 stream). */
int gastar_gen_sliding(uint32_t n, uint64_t seed, uint32_t walk_min, uint32_t walk_max,
                       uint8_t *start, uint8_t *goal);
/* Seeded grid: weights uniform in [wmin, wmax], Bernoulli(density) obstacles,
 * random monotone corridor (0,0) -> (w-1,h-1) kept passable. */
int gastar_gen_grid(uint32_t w, uint32_t h, uint64_t seed, double density, uint32_t wmin,
                    uint32_t wmax, uint8_t *weights);

#ifdef __cplusplus
}
#endif
#endif
