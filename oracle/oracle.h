/*
 * CPU oracle for the GA* search path — TEST INFRASTRUCTURE ONLY.
 *
 * This library is the checker for the GPU engine: a single-threaded host A*
 * (binary heap + open-addressing map), an exhaustive BFS over the 8-puzzle and
 * a Dijkstra/A* for weighted grids, plus move-by-move path validators.  Only
 * the test suite, the smoke check and the CPU-baseline leg of the benchmark
 * load it.  The product never links or calls it.
 *
 * What it restates (reference = michalborkowski96/cuda_a_star):
 *   - sliding-puzzle successor function  a_star_sliding_puzzle.h:84-123
 *     (move i: 0 = blank row+1, 1 = row-1, 2 = col+1, 3 = col-1, cost 1);
 *     `ref_moves` reproduces the reference's arithmetic exactly, under which
 *     moves 1 and 3 never exist (uint16 sum without 8-bit wraparound,
 *     a_star_sliding_puzzle.h:106-108);
 *   - sliding Manhattan heuristic        a_star_sliding_puzzle.h:152-163
 *     (`ref` variant sums over every cell including the blank; the
 *     admissible variant skips the blank);
 *   - grid successor function            a_star_pathfinding.h:147-209
 *     (8 moves, cost = weight of the entered cell, obstacles block entry,
 *     no corner-cutting rule);
 *   - grid heuristic                     a_star_pathfinding.h:219-221
 *     (`ref` = Manhattan; admissible = Chebyshev x minimum cell weight);
 *   - priority order                     a_star.h:55-66 (lower f, then higher g);
 *   - termination / path rebuild         a_star.h:79-83, 260-274.
 *
 * Parity pins: tests/golden holds vectors produced by compiling the
 * reference's own successor, heuristic, parser and printer functions for the
 * host (oracle/ref_harness.cu); the exhaustive 8-puzzle BFS and grid
 * Dijkstra pin the A* optimal costs independently.
 */
#ifndef GASTAR_ORACLE_H
#define GASTAR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    ORACLE_OK = 0,
    ORACLE_NO_PATH = 1,
    ORACLE_BUDGET = 2,
    ORACLE_BAD_INPUT = 3,
    ORACLE_PATH_CAP = 4,
};

enum { ORACLE_H_ADMISSIBLE = 0, ORACLE_H_REFERENCE = 1, ORACLE_H_ZERO = 2 };

typedef struct oracle_result {
    int32_t status;
    uint32_t cost;        /* optimal (or heuristic-dependent) path cost */
    uint32_t path_len;    /* number of states on the path incl. start and goal */
    uint32_t pad;
    uint64_t expansions;  /* non-stale pops that generated successors */
    uint64_t generated;   /* successors produced by the move function */
    uint64_t pushes;      /* successors that improved the table and were queued */
    double seconds;       /* wall time of the search loop */
} oracle_result;

/* ---- sliding puzzle (n = 3, 4, 5); boards are n*n bytes, row-major, 0 = blank ---- */
int oracle_sliding_successor(int n, const uint8_t *board, int move, int ref_moves,
                             uint8_t *out, uint32_t *cost);
uint32_t oracle_sliding_h(int n, const uint8_t *board, const uint8_t *goal, int heuristic);
int oracle_sliding_solvable(int n, const uint8_t *start, const uint8_t *goal);
int oracle_sliding_astar(int n, const uint8_t *start, const uint8_t *goal, int heuristic,
                         int ref_moves, uint64_t max_expansions, oracle_result *res,
                         uint8_t *path, uint32_t path_cap);
int oracle_sliding_validate(int n, const uint8_t *start, const uint8_t *goal,
                            const uint8_t *path, uint32_t len, int ref_moves, uint32_t *cost);
/* Exhaustive BFS over the 8-puzzle from `goal` (standard four moves).
 * dist has 362880 entries indexed by oracle_perm_rank9; 0xFF = unreachable. */
int oracle_bfs8(const uint8_t *goal, uint8_t *dist);
uint32_t oracle_perm_rank9(const uint8_t *board);

/* ---- weighted grid; weights w*h bytes (index y*w + x), 0 = impassable ---- */
int oracle_grid_successor(uint32_t w, uint32_t h, const uint8_t *weights, uint32_t x,
                          uint32_t y, int move, uint32_t *nx, uint32_t *ny, uint32_t *cost);
uint32_t oracle_grid_h(uint32_t x, uint32_t y, uint32_t tx, uint32_t ty, uint32_t min_weight,
                       int heuristic);
int oracle_grid_astar(uint32_t w, uint32_t h, const uint8_t *weights, uint32_t sx, uint32_t sy,
                      uint32_t tx, uint32_t ty, int heuristic, uint64_t max_expansions,
                      oracle_result *res, uint32_t *path, uint32_t path_cap);
int oracle_grid_validate(uint32_t w, uint32_t h, const uint8_t *weights, uint32_t sx,
                         uint32_t sy, uint32_t tx, uint32_t ty, const uint32_t *path,
                         uint32_t len, uint32_t *cost);

/* ---- many independent instances over host threads (CPU baseline) ----
 * Sliding: starts/goals are count*n*n bytes.  Grids: weights are concatenated,
 * offsets[i] gives the byte offset of instance i, dims[2i]=w, dims[2i+1]=h,
 * ends[4i..4i+3] = sx, sy, tx, ty.  Paths are not returned.  `threads` = 0
 * means one thread per online core. Returns the number of threads used. */
int oracle_sliding_batch(int n, uint32_t count, const uint8_t *starts, const uint8_t *goals,
                         int heuristic, int threads, oracle_result *results);
int oracle_grid_batch(uint32_t count, const uint8_t *weights, const uint64_t *offsets,
                      const uint32_t *dims, const uint32_t *ends, int heuristic, int threads,
                      oracle_result *results);

#ifdef __cplusplus
}
#endif
#endif
