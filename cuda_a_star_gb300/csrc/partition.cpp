// Host-side problem records and partition planning (see partition.h).
#include "partition.h"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "../../include/gastar.h"
#include "engine_internal.h"

namespace gastar {

namespace {

// Scheduling estimates are the expected one-block search time in ns, so that
// puzzles and grids order against each other (longest first).  Measured on
// mixed batches (16 warps, 32-wide expansion): a grid takes about 80 ns per
// cell; a 15-puzzle's mean time is about 8 ms at heuristic 22.5 and grows
// about 1.65x per 5 of heuristic, up to the ~100 ms at which its partition
// fills.  8-puzzles are small; 24-puzzles are taken as twice the 15-puzzle
// figure.
uint64_t sliding_est_ns(uint32_t n, uint32_t f0) {
    if (n == 3) return 200000ull;
    const double ms = std::min(100.0, 8.2 * std::exp(0.1002 * ((double)f0 - 22.5)));
    return (uint64_t)(ms * 1e6) * (n == 5 ? 2 : 1);
}

}  // namespace

bool make_sliding_problem(uint32_t n, const uint8_t* start, const uint8_t* goal, uint32_t heuristic,
                          uint32_t moves, Problem& p) {
    if (!valid_board(n, start) || !valid_board(n, goal)) return false;
    p = Problem();
    p.kind = n == 3 ? KIND_SLIDING3 : n == 4 ? KIND_SLIDING4 : KIND_SLIDING5;
    p.n = n;
    pack_board(n, start, p.start0, p.start1);
    pack_board(n, goal, p.goal0, p.goal1);
    p.f0 = sliding_h(n, start, goal, heuristic);
    p.unreachable = moves == GASTAR_MOVES_STANDARD && !sliding_solvable(n, start, goal);
    p.est = sliding_est_ns(n, p.f0);
    return true;
}

// Least passable (non-zero) weight, 255 if none: the minimum of w - 1 with
// obstacles (0) wrapping to 255, a plain unsigned-min reduction that the
// compiler turns into vector min instructions (a 2048^2 grid is 4 MB).
uint8_t min_passable_weight(const uint8_t* q, size_t cells) {
    uint8_t m = 255;
    for (size_t i = 0; i < cells; ++i) {
        const uint8_t t = (uint8_t)(q[i] - 1u);
        m = t < m ? t : m;
    }
    return m == 255 ? (uint8_t)255 : (uint8_t)(m + 1);
}

bool make_grid_problem(uint32_t w, uint32_t h, const uint8_t* weights, uint32_t sx, uint32_t sy,
                       uint32_t tx, uint32_t ty, uint32_t heuristic, Problem& p, bool host_copy) {
    if (!weights || !w || !h || w > 65535 || h > 65535 || sx >= w || sy >= h || tx >= w || ty >= h)
        return false;
    p = Problem();
    p.kind = KIND_GRID;
    p.W = w;
    p.H = h;
    p.start0 = (uint64_t)sy * w + sx;
    p.goal0 = (uint64_t)ty * w + tx;
    const size_t cells = (size_t)w * h;
    p.est = 80ull * cells;
    if (!host_copy) return true;
    p.weights.assign(weights, weights + cells);
    set_grid_minw(p, min_passable_weight(weights, cells), heuristic);
    return true;
}

void set_grid_minw(Problem& p, uint32_t minw, uint32_t heuristic) {
    p.minw = minw;
    const uint32_t sx = (uint32_t)(p.start0 % p.W), sy = (uint32_t)(p.start0 / p.W);
    const uint32_t tx = (uint32_t)(p.goal0 % p.W), ty = (uint32_t)(p.goal0 / p.W);
    p.f0 = grid_h(sx, sy, tx, ty, minw, heuristic);
}

PartPlan plan_partition(const Problem& p, const PartConfig& c) {
    PartPlan pl;
    const float lf = std::min(0.95f, std::max(0.1f, c.load_factor));
    uint64_t entries, table_bytes;
    if (p.kind == KIND_GRID) {
        const uint64_t cells = (uint64_t)p.W * p.H;
        pl.table_words = cells;
        pl.table_limit = ~0ull;
        table_bytes = cells * 8;
        entries = std::max<uint64_t>(1 << 16, cells / 2) << (2 * c.retry_level);
        pl.path_words = std::max<uint64_t>(1024, 4ull * (p.W + p.H)) << c.retry_level;
    } else {
        uint64_t states = c.sliding_states ? c.sliding_states : (p.n == 3 ? 181440ull : (1ull << 20));
        if (p.n != 3) states <<= 2 * c.retry_level;
        const uint64_t slots = next_pow2((uint64_t)((double)states / lf) + 1);
        const uint32_t sw = key_words(p.kind) == 1 ? 2 : 4;
        pl.table_words = slots * sw;
        pl.table_mask = slots - 1;
        pl.table_limit = (uint64_t)((double)slots * lf);
        table_bytes = pl.table_words * 8;
        entries = states;
        pl.path_words = (512ull * key_words(p.kind)) << c.retry_level;
    }
    const uint64_t per_heap = (entries + c.warps - 1) / c.warps;
    pl.heap_cap = (uint32_t)std::max<uint64_t>(2 * c.heap_snodes, (per_heap * 2 + 31) / 32);
    const uint64_t hdr_end = table_bytes + (uint64_t)c.warps * 8;
    pl.heap_off = (hdr_end + 255) & ~255ull;
    const uint64_t heap_bytes = (uint64_t)c.warps * (pl.heap_cap + 1) * 32 * entry_bytes(p.kind);
    uint64_t end = pl.heap_off + heap_bytes;
    if (c.buckets) {  // as many pages per warp as the heap has nodes
        pl.bq_pages = pl.heap_cap;
        pl.bq_off = (end + 255) & ~255ull;
        end = pl.bq_off + bucket_area_bytes(c.warps, pl.bq_pages, entry_bytes(p.kind));
    }
    if (p.kind != KIND_GRID && c.claim_list) {
        // Claims stop within two iterations past the limit; every warp may
        // leave one chunk partly unused (as the plain engine's list).
        pl.touched_cap = pl.table_limit + 2ull * c.warps * c.ew * max_neighbours(p.kind) +
                         (uint64_t)c.warps * kTouchedChunk + 16;
        pl.touched_off = (end + 255) & ~255ull;
        end = pl.touched_off + pl.touched_cap * 4;
    }
    if (p.kind == KIND_GRID && c.own_weights) {
        pl.weights_off = (end + 255) & ~255ull;
        end = pl.weights_off + (uint64_t)p.W * p.H;
    }
    pl.bytes = (end + 255) & ~255ull;
    return pl;
}

void fill_desc(InstDesc& d, const Problem& p, const PartConfig& c, const PartPlan& pl, char* base,
               const uint8_t* d_weights, InstCtl* ctl, unsigned long long* touched_count) {
    std::memset(&d, 0, sizeof(d));
    d.kind = p.kind;
    d.heuristic = c.heuristic;
    d.moves = c.moves;
    d.n = p.n;
    d.start0 = p.start0;
    d.start1 = p.start1;
    d.goal0 = p.goal0;
    d.goal1 = p.goal1;
    d.W = p.W;
    d.H = p.H;
    d.minw = p.minw;
    d.f0 = p.f0;
    d.table = reinterpret_cast<unsigned long long*>(base);
    d.table_words = pl.table_words;
    d.table_mask = pl.table_mask;
    d.table_limit = pl.table_limit;
    d.max_probe = 4096;
    d.heaps = c.warps;
    d.heap_hdr = reinterpret_cast<uint32_t*>(base + pl.table_words * 8);
    d.heap_nodes = base + pl.heap_off;
    if (pl.bq_pages) {
        d.bq_base = base + pl.bq_off;
        d.bq_pages = pl.bq_pages;
    }
    d.heap_cap = pl.heap_cap;
    d.ew = c.ew;
    d.max_exp = c.max_exp;
    d.timeout_ns = (uint64_t)c.timeout_ms * 1000000ull;
    d.delta = p.kind == KIND_GRID ? c.delta_grid : 0;
    d.ctl = ctl;
    if (p.kind == KIND_GRID)
        d.weights = c.own_weights ? reinterpret_cast<const uint8_t*>(base + pl.weights_off) : d_weights;
    if (pl.touched_cap && touched_count) {
        d.touched = reinterpret_cast<uint32_t*>(base + pl.touched_off);
        d.touched_count = touched_count;
        d.touched_cap = pl.touched_cap;
        d.prev_slot_words = key_words(p.kind) == 1 ? 2 : 4;
        d.clear_either = 1;  // the list always refers to this partition's table
    }
}

}  // namespace gastar
