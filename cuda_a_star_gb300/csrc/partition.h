// Host-side problem records and per-instance partition planning shared by the
// batched and the served engines.
#pragma once

#include <cstdint>
#include <vector>

#include "engine_types.h"

namespace gastar {

// One instance as the host keeps it.
struct Problem {
    uint32_t kind = 0, n = 0;
    uint64_t start0 = 0, start1 = 0, goal0 = 0, goal1 = 0;
    uint32_t W = 0, H = 0, minw = 0, f0 = 0;
    bool unreachable = false;      // other parity class of the standard sliding moves
    std::vector<uint8_t> weights;  // grid, host copy (served requests)
    const uint8_t* d_weights = nullptr;  // grid, device copy (batched instances; owned by the batch)
    uint64_t est = 0;              // expected one-block search time in ns
};

// Launch order inside a persistent launch (longest processing time first):
// 15- and 24-puzzles first -- their time is not predictable from the start
// state, but their partition bounds it (about 100 ms on one block before it
// fills), so the long ones among them start early instead of forming the
// tail -- then by expected time, largest first, so that the small grids fill
// the end.
inline bool sched_before(const Problem& a, const Problem& b) {
    const bool ua = a.kind != KIND_GRID && a.n >= 4, ub = b.kind != KIND_GRID && b.n >= 4;
    if (ua != ub) return ua;
    return a.est > b.est;
}

// Sizing knobs of a partition.
struct PartConfig {
    uint32_t warps = 8, ew = 32;
    float load_factor = 0.75f;
    uint32_t heuristic = 0, moves = 0, delta_grid = 0;
    uint64_t sliding_states = 0;  // 0 = by class
    uint64_t max_exp = 0;
    uint32_t timeout_ms = 0;
    uint32_t retry_level = 0;     // capacities scale by 4^retry_level
    uint32_t heap_snodes = kHeapSmemNodes;  // heap nodes below this index live in shared memory
    bool buckets = false;         // bucket front in front of the warp-heaps
    bool own_weights = false;     // grid weights live inside the partition
    bool claim_list = false;      // puzzles: record claimed slots so that the next search
                                  // in the same partition clears only those
};

// Byte layout of one partition:
// table | heap headers | heap nodes | bucket area | claim list | weights.
struct PartPlan {
    uint64_t table_words = 0, table_mask = 0, table_limit = 0;
    uint32_t heap_cap = 0;
    uint64_t heap_off = 0, weights_off = 0, bytes = 0;
    uint64_t bq_off = 0;          // bucket area (pages, links, free stacks)
    uint32_t bq_pages = 0;        // pages per warp (0 = no buckets)
    uint64_t path_words = 0;      // path-arena share
    uint64_t touched_off = 0;     // claim list (u32 word offsets of claimed slots)
    uint64_t touched_cap = 0;     // its capacity in entries (0 = no claim list)
};

bool make_sliding_problem(uint32_t n, const uint8_t* start, const uint8_t* goal, uint32_t heuristic,
                          uint32_t moves, Problem& p);
// With host_copy false the weights are neither copied nor scanned: the caller
// places them (on the device) and sets the least weight with set_grid_minw.
bool make_grid_problem(uint32_t w, uint32_t h, const uint8_t* weights, uint32_t sx, uint32_t sy,
                       uint32_t tx, uint32_t ty, uint32_t heuristic, Problem& p, bool host_copy = true);
// Least passable weight of a grid problem (255: none) and the start's f.
void set_grid_minw(Problem& p, uint32_t minw, uint32_t heuristic);
PartPlan plan_partition(const Problem& p, const PartConfig& c);
// Fills an instance descriptor for a partition placed at `base` (256-byte
// aligned).  `d_weights` is used for grids unless the partition owns them.
// `touched_count` is the claim list's length word when the plan has a claim
// list: above the list's capacity (the value the host sets for memory whose
// contents are unknown) it makes the next search clear the whole table.
void fill_desc(InstDesc& d, const Problem& p, const PartConfig& c, const PartPlan& plan, char* base,
               const uint8_t* d_weights, InstCtl* ctl, unsigned long long* touched_count = nullptr);

}  // namespace gastar
