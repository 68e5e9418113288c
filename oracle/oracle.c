/*
 * CPU oracle for the GA* search path — TEST INFRASTRUCTURE ONLY (see oracle.h).
 * Only tests, the smoke check and the benchmark's CPU-baseline leg load this.
 *
 * Every function cites the reference (michalborkowski96/cuda_a_star) file:line
 * whose behaviour it restates.  Plain C11 + pthreads; no architecture-specific
 * code, so it builds and gives identical results on x86_64 and aarch64.
 */
#include "oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

typedef unsigned __int128 u128;

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static inline uint64_t mix64(uint64_t x) { /* SplitMix64 finaliser (Steele et al. 2014) */
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebULL;
    x ^= x >> 31;
    return x;
}

/* ------------------------------------------------------------------------- */
/* Sliding puzzle move semantics                                              */
/* ------------------------------------------------------------------------- */

/* Move i moves the blank by (drow, dcol): 0:(+1,0) 1:(-1,0) 2:(0,+1) 3:(0,-1)
 * (a_star_sliding_puzzle.h:88-105). */
static const int SL_DR[4] = {1, -1, 0, 0};
static const int SL_DC[4] = {0, 0, 1, -1};

/* Returns the blank's new cell for move `move`, or -1 when the move does not
 * exist.  With ref_moves the reference's arithmetic is reproduced: the
 * unsigned-char delta 0xff is added to the blank coordinate in a uint16 without
 * wrapping, so the sum is >= 255 and moves 1 and 3 never exist
 * (a_star_sliding_puzzle.h:86-111). */
static int sl_target_cell(int n, int blank, int move, int ref_moves) {
    int r = blank / n, c = blank % n;
    if (ref_moves) {
        unsigned dx = (move == 0) ? 1u : (move == 1 ? 0xffu : 0u);
        unsigned dy = (move == 2) ? 1u : (move == 3 ? 0xffu : 0u);
        uint16_t nr = (uint16_t)((unsigned)r + dx);
        uint16_t nc = (uint16_t)((unsigned)c + dy);
        if (nr >= n || nc >= n) return -1;
        return nr * n + nc;
    }
    int nr = r + SL_DR[move], nc = c + SL_DC[move];
    if (nr < 0 || nr >= n || nc < 0 || nc >= n) return -1;
    return nr * n + nc;
}

static int sl_find_blank(int n, const uint8_t *b) {
    for (int i = 0; i < n * n; ++i)
        if (b[i] == 0) return i;
    return -1;
}

static int sl_valid_board(int n, const uint8_t *b) {
    if (n < 2 || n > 5) return 0;
    uint32_t seen = 0;
    for (int i = 0; i < n * n; ++i) {
        if (b[i] >= n * n) return 0;
        if (seen & (1u << b[i])) return 0;
        seen |= 1u << b[i];
    }
    return 1;
}

int oracle_sliding_successor(int n, const uint8_t *board, int move, int ref_moves,
                             uint8_t *out, uint32_t *cost) {
    /* a_star_sliding_puzzle.h:84-123: cost 1, tile at the target cell moves
     * into the blank's cell, blank moves to the target cell. */
    *cost = 1;
    int blank = sl_find_blank(n, board);
    if (blank < 0 || move < 0 || move > 3) return 0;
    int q = sl_target_cell(n, blank, move, ref_moves);
    if (q < 0) return 0;
    memcpy(out, board, (size_t)n * n);
    out[blank] = board[q];
    out[q] = 0;
    return 1;
}

static void sl_goal_tables(int n, const uint8_t *goal, uint8_t *gr, uint8_t *gc) {
    /* set_manhattan_heuristic_target: goal row/col of every tile value
     * (a_star_sliding_puzzle.h:130-142). */
    for (int i = 0; i < n * n; ++i) {
        gr[goal[i]] = (uint8_t)(i / n);
        gc[goal[i]] = (uint8_t)(i % n);
    }
}

uint32_t oracle_sliding_h(int n, const uint8_t *board, const uint8_t *goal, int heuristic) {
    /* a_star_sliding_puzzle.h:152-163 sums |goal_row - row| + |goal_col - col|
     * over every cell, the blank included (ORACLE_H_REFERENCE).  The admissible
     * variant leaves the blank out. */
    if (heuristic == ORACLE_H_ZERO) return 0;
    uint8_t gr[32], gc[32];
    sl_goal_tables(n, goal, gr, gc);
    uint32_t s = 0;
    for (int i = 0; i < n * n; ++i) {
        int t = board[i];
        if (t == 0 && heuristic == ORACLE_H_ADMISSIBLE) continue;
        int dr = (int)gr[t] - i / n, dc = (int)gc[t] - i % n;
        s += (uint32_t)(abs(dr) + abs(dc));
    }
    return s;
}

static uint32_t sl_invariant(int n, const uint8_t *b) {
    uint32_t inv = 0;
    for (int i = 0; i < n * n; ++i) {
        if (!b[i]) continue;
        for (int j = i + 1; j < n * n; ++j)
            if (b[j] && b[j] < b[i]) ++inv;
    }
    if ((n & 1) == 0) inv += (uint32_t)(sl_find_blank(n, b) / n);
    return inv & 1u;
}

int oracle_sliding_solvable(int n, const uint8_t *start, const uint8_t *goal) {
    /* Standard four-move puzzle: two states are connected iff this parity
     * invariant agrees (odd n: tile inversions; even n: inversions + blank row). */
    if (!sl_valid_board(n, start) || !sl_valid_board(n, goal)) return 0;
    return sl_invariant(n, start) == sl_invariant(n, goal);
}

/* 5 bits per tile, tile at cell i in bits [5i, 5i+5): fits n <= 5. */
static u128 sl_pack(int n, const uint8_t *b) {
    u128 k = 0;
    for (int i = 0; i < n * n; ++i) k |= (u128)b[i] << (5 * i);
    return k;
}
static inline int sl_get(u128 k, int i) { return (int)((k >> (5 * i)) & 31u); }
static inline u128 sl_move_blank(u128 k, int blank, int q) {
    u128 t = (u128)sl_get(k, q);
    k &= ~((u128)31u << (5 * q));   /* blank (0) now at q */
    k |= t << (5 * blank);          /* tile moves into the old blank cell */
    return k;
}
static void sl_unpack(int n, u128 k, uint8_t *b) {
    for (int i = 0; i < n * n; ++i) b[i] = (uint8_t)sl_get(k, i);
}

/* ---- open-addressing map u128 -> (g, parent move) ---- */
typedef struct {
    uint64_t lo, hi; /* hi == ~0 marks an empty slot (bits 125..127 are never set) */
    uint32_t g;
    uint8_t move;
} sl_slot;

typedef struct {
    sl_slot *s;
    uint64_t cap, used;
} sl_map;

static uint64_t sl_hash(uint64_t lo, uint64_t hi) { return mix64(lo ^ mix64(hi + 0x9e3779b97f4a7c15ULL)); }

static int sl_map_init(sl_map *m, uint64_t cap) {
    m->cap = cap;
    m->used = 0;
    m->s = (sl_slot *)malloc(sizeof(sl_slot) * cap);
    if (!m->s) return 0;
    for (uint64_t i = 0; i < cap; ++i) m->s[i].hi = ~0ULL;
    return 1;
}

static sl_slot *sl_map_find(sl_map *m, uint64_t lo, uint64_t hi, int *created) {
    uint64_t mask = m->cap - 1, i = sl_hash(lo, hi) & mask;
    for (;;) {
        sl_slot *s = &m->s[i];
        if (s->hi == ~0ULL) {
            s->lo = lo;
            s->hi = hi;
            s->g = 0xffffffffu;
            s->move = 0xff;
            ++m->used;
            *created = 1;
            return s;
        }
        if (s->lo == lo && s->hi == hi) {
            *created = 0;
            return s;
        }
        i = (i + 1) & mask;
    }
}

static sl_slot *sl_map_get(const sl_map *m, uint64_t lo, uint64_t hi) {
    uint64_t mask = m->cap - 1, i = sl_hash(lo, hi) & mask;
    for (;;) {
        sl_slot *s = &m->s[i];
        if (s->hi == ~0ULL) return NULL;
        if (s->lo == lo && s->hi == hi) return s;
        i = (i + 1) & mask;
    }
}

static int sl_map_grow(sl_map *m) {
    sl_map nm;
    if (!sl_map_init(&nm, m->cap * 2)) return 0;
    for (uint64_t i = 0; i < m->cap; ++i) {
        if (m->s[i].hi == ~0ULL) continue;
        int c;
        sl_slot *d = sl_map_find(&nm, m->s[i].lo, m->s[i].hi, &c);
        d->g = m->s[i].g;
        d->move = m->s[i].move;
    }
    free(m->s);
    *m = nm;
    return 1;
}

/* ---- binary heap ordered like QueueValue (a_star.h:58-63): lower f first,
 * equal f -> higher g first ---- */
typedef struct {
    uint32_t f, g;
    uint64_t lo, hi;
} sl_entry;

typedef struct {
    sl_entry *a;
    uint64_t n, cap;
} sl_heap;

static inline int sl_before(const sl_entry *x, const sl_entry *y) {
    return x->f < y->f || (x->f == y->f && x->g > y->g);
}

static int sl_heap_push(sl_heap *h, sl_entry e) {
    if (h->n == h->cap) {
        uint64_t nc = h->cap ? h->cap * 2 : 1024;
        sl_entry *na = (sl_entry *)realloc(h->a, nc * sizeof(sl_entry));
        if (!na) return 0;
        h->a = na;
        h->cap = nc;
    }
    uint64_t i = h->n++;
    while (i) {
        uint64_t p = (i - 1) >> 1;
        if (!sl_before(&e, &h->a[p])) break;
        h->a[i] = h->a[p];
        i = p;
    }
    h->a[i] = e;
    return 1;
}

static sl_entry sl_heap_pop(sl_heap *h) {
    sl_entry top = h->a[0], last = h->a[--h->n];
    uint64_t i = 0;
    for (;;) {
        uint64_t l = 2 * i + 1, r = l + 1, b = i;
        const sl_entry *best = &last;
        if (l < h->n && sl_before(&h->a[l], best)) { b = l; best = &h->a[l]; }
        if (r < h->n && sl_before(&h->a[r], best)) { b = r; best = &h->a[r]; }
        if (b == i) break;
        h->a[i] = h->a[b];
        i = b;
    }
    if (h->n) h->a[i] = last;
    return top;
}

static int sl_inverse_move(int m) { return m ^ 1; } /* 0<->1, 2<->3 */

int oracle_sliding_astar(int n, const uint8_t *start, const uint8_t *goal, int heuristic,
                         int ref_moves, uint64_t max_expansions, oracle_result *res,
                         uint8_t *path, uint32_t path_cap) {
    /* Single-thread A* with the reference's priority order and goal test at pop
     * (a_star.h:58-63, 79-83), reopening of improved states (fancy_hashmap.h:32-81
     * UPDATED semantics) and parent-chain path rebuild (a_star.h:268-281). */
    memset(res, 0, sizeof(*res));
    if (!sl_valid_board(n, start) || !sl_valid_board(n, goal)) {
        res->status = ORACLE_BAD_INPUT;
        return res->status;
    }
    double t0 = now_s();
    const int cells = n * n;
    uint8_t gr[32], gc[32];
    sl_goal_tables(n, goal, gr, gc);
    /* md[t][p]: Manhattan distance of tile t placed at cell p. */
    uint8_t md[32][32];
    for (int t = 0; t < cells; ++t)
        for (int p = 0; p < cells; ++p)
            md[t][p] = (uint8_t)(abs((int)gr[t] - p / n) + abs((int)gc[t] - p % n));
    const int blank_counts = heuristic == ORACLE_H_REFERENCE;
    const int zero_h = heuristic == ORACLE_H_ZERO;

    u128 sk = sl_pack(n, start), gk = sl_pack(n, goal);
    sl_map map;
    sl_heap heap = {0};
    if (!sl_map_init(&map, 1u << 16)) {
        res->status = ORACLE_BAD_INPUT;
        return res->status;
    }
    int created;
    sl_slot *s0 = sl_map_find(&map, (uint64_t)sk, (uint64_t)(sk >> 64), &created);
    s0->g = 0;
    s0->move = 0xff;
    uint32_t h0 = zero_h ? 0 : oracle_sliding_h(n, start, goal, heuristic);
    sl_heap_push(&heap, (sl_entry){h0, 0, (uint64_t)sk, (uint64_t)(sk >> 64)});

    int found = 0;
    uint32_t best = 0;
    while (heap.n) {
        sl_entry e = sl_heap_pop(&heap);
        sl_slot *se = sl_map_get(&map, e.lo, e.hi);
        if (se->g < e.g) continue; /* stale (lazy deletion) */
        u128 k = (u128)e.lo | ((u128)e.hi << 64);
        if (k == gk) {
            found = 1;
            best = e.g;
            break;
        }
        if (max_expansions && res->expansions >= max_expansions) {
            res->status = ORACLE_BUDGET;
            break;
        }
        ++res->expansions;
        int blank = 0;
        while (sl_get(k, blank) != 0) ++blank;
        uint32_t h = e.f - e.g;
        for (int m = 0; m < 4; ++m) {
            int q = sl_target_cell(n, blank, m, ref_moves);
            if (q < 0) continue;
            ++res->generated;
            int t = sl_get(k, q);
            uint32_t nh = zero_h ? 0
                                 : h + md[t][blank] - md[t][q] +
                                       (blank_counts ? (uint32_t)md[0][q] - md[0][blank] : 0);
            u128 nk = sl_move_blank(k, blank, q);
            uint32_t ng = e.g + 1;
            if (map.used * 2 >= map.cap && !sl_map_grow(&map)) {
                res->status = ORACLE_BAD_INPUT;
                goto done;
            }
            sl_slot *ns = sl_map_find(&map, (uint64_t)nk, (uint64_t)(nk >> 64), &created);
            if (ng < ns->g) {
                ns->g = ng;
                ns->move = (uint8_t)m;
                ++res->pushes;
                sl_heap_push(&heap, (sl_entry){ng + nh, ng, (uint64_t)nk, (uint64_t)(nk >> 64)});
            }
        }
    }
    if (res->status == ORACLE_BUDGET) goto done;
    if (!found) {
        res->status = ORACLE_NO_PATH;
        goto done;
    }
    res->cost = best;
    res->path_len = best + 1;
    if (path && path_cap) {
        if (best + 1 > path_cap) {
            res->status = ORACLE_PATH_CAP;
            goto done;
        }
        u128 k = gk;
        for (int64_t i = best; i >= 0; --i) {
            sl_unpack(n, k, path + (size_t)i * cells);
            if (i == 0) break;
            sl_slot *s = sl_map_get(&map, (uint64_t)k, (uint64_t)(k >> 64));
            int blank = 0;
            while (sl_get(k, blank) != 0) ++blank;
            int q = sl_target_cell(n, blank, sl_inverse_move(s->move), 0);
            k = sl_move_blank(k, blank, q);
        }
    }
    res->status = ORACLE_OK;
done:
    res->seconds = now_s() - t0;
    free(map.s);
    free(heap.a);
    return res->status;
}

int oracle_sliding_validate(int n, const uint8_t *start, const uint8_t *goal,
                            const uint8_t *path, uint32_t len, int ref_moves, uint32_t *cost) {
    /* Move-by-move check: each consecutive pair must be related by one of the
     * successor function's moves (a_star_sliding_puzzle.h:84-123). */
    const int cells = n * n;
    *cost = 0;
    if (len == 0) return 0;
    if (memcmp(path, start, cells) || memcmp(path + (size_t)(len - 1) * cells, goal, cells)) return 0;
    uint8_t tmp[32];
    for (uint32_t i = 0; i + 1 < len; ++i) {
        int ok = 0;
        for (int m = 0; m < 4 && !ok; ++m) {
            uint32_t c;
            if (oracle_sliding_successor(n, path + (size_t)i * cells, m, ref_moves, tmp, &c) &&
                !memcmp(tmp, path + (size_t)(i + 1) * cells, cells)) {
                ok = 1;
                *cost += c;
            }
        }
        if (!ok) return 0;
    }
    return 1;
}

uint32_t oracle_perm_rank9(const uint8_t *b) {
    /* Lehmer-code rank of a permutation of 0..8. */
    static const uint32_t fact[9] = {1, 1, 2, 6, 24, 120, 720, 5040, 40320};
    uint32_t r = 0;
    for (int i = 0; i < 9; ++i) {
        uint32_t smaller = 0;
        for (int j = i + 1; j < 9; ++j)
            if (b[j] < b[i]) ++smaller;
        r += smaller * fact[8 - i];
    }
    return r;
}

int oracle_bfs8(const uint8_t *goal, uint8_t *dist) {
    /* Exhaustive breadth-first search from the goal with the standard four moves:
     * the distance of every reachable 8-puzzle state (181,440 of the 362,880). */
    if (!sl_valid_board(3, goal)) return -1;
    memset(dist, 0xff, 362880);
    uint8_t (*queue)[9] = malloc(181440 * 9 + 9);
    if (!queue) return -1;
    uint32_t head = 0, tail = 0;
    memcpy(queue[tail++], goal, 9);
    dist[oracle_perm_rank9(goal)] = 0;
    while (head < tail) {
        uint8_t *b = queue[head++];
        uint8_t d = dist[oracle_perm_rank9(b)];
        for (int m = 0; m < 4; ++m) {
            uint8_t nb[9];
            uint32_t c;
            if (!oracle_sliding_successor(3, b, m, 0, nb, &c)) continue;
            uint32_t r = oracle_perm_rank9(nb);
            if (dist[r] != 0xff) continue;
            dist[r] = (uint8_t)(d + 1);
            memcpy(queue[tail++], nb, 9);
        }
    }
    free(queue);
    return (int)tail;
}

/* ------------------------------------------------------------------------- */
/* Weighted grid                                                              */
/* ------------------------------------------------------------------------- */

/* Move i: 0:(+1,0) 1:(-1,0) 2:(0,+1) 3:(0,-1) 4:(+1,+1) 5:(+1,-1) 6:(-1,+1)
 * 7:(-1,-1) in (x, y) (a_star_pathfinding.h:150-183). */
static const int GR_DX[8] = {1, -1, 0, 0, 1, 1, -1, -1};
static const int GR_DY[8] = {0, 0, 1, -1, 1, -1, 1, -1};

int oracle_grid_successor(uint32_t w, uint32_t h, const uint8_t *weights, uint32_t x,
                          uint32_t y, int move, uint32_t *nx, uint32_t *ny, uint32_t *cost) {
    /* a_star_pathfinding.h:147-209: off-board and obstacle cells do not exist;
     * the cost is the entered cell's weight.  The reference narrows the new
     * coordinates to 8 bits (185-186), which is exact for boards up to 255
     * cells a side; this restatement keeps full-width coordinates. */
    if (move < 0 || move > 7) return 0;
    int64_t X = (int64_t)x + GR_DX[move], Y = (int64_t)y + GR_DY[move];
    if (X < 0 || Y < 0 || X >= (int64_t)w || Y >= (int64_t)h) return 0;
    uint8_t wt = weights[(size_t)Y * w + (size_t)X];
    if (!wt) return 0;
    *nx = (uint32_t)X;
    *ny = (uint32_t)Y;
    *cost = wt;
    return 1;
}

uint32_t oracle_grid_h(uint32_t x, uint32_t y, uint32_t tx, uint32_t ty, uint32_t min_weight,
                       int heuristic) {
    /* ORACLE_H_REFERENCE: |tx-x| + |ty-y| (a_star_pathfinding.h:219-221).
     * ORACLE_H_ADMISSIBLE: max(|dx|,|dy|) * minimum cell weight, a lower bound
     * for 8-connected moves that each cost at least min_weight. */
    uint32_t dx = x > tx ? x - tx : tx - x, dy = y > ty ? y - ty : ty - y;
    if (heuristic == ORACLE_H_REFERENCE) return dx + dy;
    if (heuristic == ORACLE_H_ZERO) return 0;
    return (dx > dy ? dx : dy) * min_weight;
}

typedef struct {
    uint32_t f, g, cell, pad;
} gr_entry;

typedef struct {
    gr_entry *a;
    uint64_t n, cap;
} gr_heap;

static inline int gr_before(const gr_entry *x, const gr_entry *y) {
    return x->f < y->f || (x->f == y->f && x->g > y->g);
}

static int gr_heap_push(gr_heap *h, gr_entry e) {
    if (h->n == h->cap) {
        uint64_t nc = h->cap ? h->cap * 2 : 4096;
        gr_entry *na = (gr_entry *)realloc(h->a, nc * sizeof(gr_entry));
        if (!na) return 0;
        h->a = na;
        h->cap = nc;
    }
    uint64_t i = h->n++;
    while (i) {
        uint64_t p = (i - 1) >> 1;
        if (!gr_before(&e, &h->a[p])) break;
        h->a[i] = h->a[p];
        i = p;
    }
    h->a[i] = e;
    return 1;
}

static gr_entry gr_heap_pop(gr_heap *h) {
    gr_entry top = h->a[0], last = h->a[--h->n];
    uint64_t i = 0;
    for (;;) {
        uint64_t l = 2 * i + 1, r = l + 1, b = i;
        const gr_entry *best = &last;
        if (l < h->n && gr_before(&h->a[l], best)) { b = l; best = &h->a[l]; }
        if (r < h->n && gr_before(&h->a[r], best)) { b = r; best = &h->a[r]; }
        if (b == i) break;
        h->a[i] = h->a[b];
        i = b;
    }
    if (h->n) h->a[i] = last;
    return top;
}

int oracle_grid_astar(uint32_t w, uint32_t h, const uint8_t *weights, uint32_t sx, uint32_t sy,
                      uint32_t tx, uint32_t ty, int heuristic, uint64_t max_expansions,
                      oracle_result *res, uint32_t *path, uint32_t path_cap) {
    /* Dense-array A* on the reference's 8-connected move set
     * (a_star_pathfinding.h:147-221) with the reference's priority order and
     * goal test at pop (a_star.h:58-63, 79-83). */
    /* Like the reference, the start is expanded even when it is an obstacle
     * (only entering a cell is checked, a_star_pathfinding.h:196), and an
     * impassable goal is unreachable unless it is the start. */
    memset(res, 0, sizeof(*res));
    if (!w || !h || sx >= w || sy >= h || tx >= w || ty >= h) {
        res->status = ORACLE_BAD_INPUT;
        return res->status;
    }
    double t0 = now_s();
    const size_t cells = (size_t)w * h;
    uint32_t minw = 255;
    for (size_t i = 0; i < cells; ++i)
        if (weights[i] && weights[i] < minw) minw = weights[i];
    uint32_t *g = (uint32_t *)malloc(cells * sizeof(uint32_t));
    uint8_t *par = (uint8_t *)malloc(cells);
    gr_heap heap = {0};
    if (!g || !par) {
        free(g);
        free(par);
        res->status = ORACLE_BAD_INPUT;
        return res->status;
    }
    memset(g, 0xff, cells * sizeof(uint32_t));
    const uint32_t start = sy * w + sx, goal = ty * w + tx;
    g[start] = 0;
    par[start] = 0xff;
    gr_heap_push(&heap, (gr_entry){oracle_grid_h(sx, sy, tx, ty, minw, heuristic), 0, start, 0});
    int found = 0;
    uint32_t best = 0;
    while (heap.n) {
        gr_entry e = gr_heap_pop(&heap);
        if (g[e.cell] < e.g) continue;
        if (e.cell == goal) {
            found = 1;
            best = e.g;
            break;
        }
        if (max_expansions && res->expansions >= max_expansions) {
            res->status = ORACLE_BUDGET;
            break;
        }
        ++res->expansions;
        uint32_t x = e.cell % w, y = e.cell / w;
        for (int m = 0; m < 8; ++m) {
            uint32_t nx, ny, c;
            if (!oracle_grid_successor(w, h, weights, x, y, m, &nx, &ny, &c)) continue;
            ++res->generated;
            uint32_t nc = ny * w + nx, ng = e.g + c;
            if (ng < g[nc]) {
                g[nc] = ng;
                par[nc] = (uint8_t)m;
                ++res->pushes;
                gr_heap_push(&heap,
                             (gr_entry){ng + oracle_grid_h(nx, ny, tx, ty, minw, heuristic), ng, nc, 0});
            }
        }
    }
    if (res->status == ORACLE_BUDGET) goto done;
    if (!found) {
        res->status = ORACLE_NO_PATH;
        goto done;
    }
    res->cost = best;
    {
        uint32_t len = 1;
        for (uint32_t c = goal; c != start; ++len) {
            int m = par[c];
            c = (uint32_t)((int64_t)c - GR_DX[m] - (int64_t)GR_DY[m] * w);
        }
        res->path_len = len;
        if (path && path_cap) {
            if (len > path_cap) {
                res->status = ORACLE_PATH_CAP;
                goto done;
            }
            uint32_t c = goal;
            for (int64_t i = len - 1; i >= 0; --i) {
                path[i] = c;
                if (i == 0) break;
                int m = par[c];
                c = (uint32_t)((int64_t)c - GR_DX[m] - (int64_t)GR_DY[m] * w);
            }
        }
    }
    res->status = ORACLE_OK;
done:
    res->seconds = now_s() - t0;
    free(g);
    free(par);
    free(heap.a);
    return res->status;
}

int oracle_grid_validate(uint32_t w, uint32_t h, const uint8_t *weights, uint32_t sx,
                         uint32_t sy, uint32_t tx, uint32_t ty, const uint32_t *path,
                         uint32_t len, uint32_t *cost) {
    /* Move-by-move check against a_star_pathfinding.h:147-209: neighbours in the
     * 8-neighbourhood, entered cells passable, cost = sum of entered weights. */
    *cost = 0;
    if (len == 0 || path[0] != sy * w + sx || path[len - 1] != ty * w + tx) return 0;
    for (uint32_t i = 0; i + 1 < len; ++i) {
        if (path[i] >= w * h || path[i + 1] >= w * h) return 0;
        int64_t x0 = path[i] % w, y0 = path[i] / w, x1 = path[i + 1] % w, y1 = path[i + 1] / w;
        int64_t dx = x1 - x0, dy = y1 - y0;
        if ((dx == 0 && dy == 0) || dx < -1 || dx > 1 || dy < -1 || dy > 1) return 0;
        uint8_t wt = weights[path[i + 1]];
        if (!wt) return 0;
        *cost += wt;
    }
    return 1;
}

/* ------------------------------------------------------------------------- */
/* Many instances over host threads                                           */
/* ------------------------------------------------------------------------- */

typedef struct {
    int kind; /* 0 sliding, 1 grid */
    int n, heuristic;
    uint32_t count;
    const uint8_t *starts, *goals;
    const uint8_t *weights;
    const uint64_t *offsets;
    const uint32_t *dims, *ends;
    oracle_result *results;
    uint32_t next;
} batch_job;

static void *batch_worker(void *arg) {
    batch_job *j = (batch_job *)arg;
    for (;;) {
        uint32_t i = __atomic_fetch_add(&j->next, 1u, __ATOMIC_RELAXED);
        if (i >= j->count) break;
        if (j->kind == 0) {
            size_t c = (size_t)j->n * j->n;
            oracle_sliding_astar(j->n, j->starts + i * c, j->goals + i * c, j->heuristic, 0, 0,
                                 &j->results[i], NULL, 0);
        } else {
            oracle_grid_astar(j->dims[2 * i], j->dims[2 * i + 1], j->weights + j->offsets[i],
                              j->ends[4 * i], j->ends[4 * i + 1], j->ends[4 * i + 2],
                              j->ends[4 * i + 3], j->heuristic, 0, &j->results[i], NULL, 0);
        }
    }
    return NULL;
}

static int run_batch(batch_job *j, int threads) {
    if (threads <= 0) {
        long c = sysconf(_SC_NPROCESSORS_ONLN);
        threads = c > 0 ? (int)c : 1;
    }
    if ((uint32_t)threads > j->count && j->count) threads = (int)j->count;
    if (threads < 1) threads = 1;
    pthread_t *tid = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
    for (int t = 0; t < threads; ++t) pthread_create(&tid[t], NULL, batch_worker, j);
    for (int t = 0; t < threads; ++t) pthread_join(tid[t], NULL);
    free(tid);
    return threads;
}

int oracle_sliding_batch(int n, uint32_t count, const uint8_t *starts, const uint8_t *goals,
                         int heuristic, int threads, oracle_result *results) {
    batch_job j = {0, n, heuristic, count, starts, goals, NULL, NULL, NULL, NULL, results, 0};
    return run_batch(&j, threads);
}

int oracle_grid_batch(uint32_t count, const uint8_t *weights, const uint64_t *offsets,
                      const uint32_t *dims, const uint32_t *ends, int heuristic, int threads,
                      oracle_result *results) {
    batch_job j = {1, 0, heuristic, count, NULL, NULL, weights, offsets, dims, ends, results, 0};
    return run_batch(&j, threads);
}
