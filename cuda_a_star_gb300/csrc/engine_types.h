// Host/device shared descriptors of the GA* engine.
#pragma once

#include <cstddef>
#include <cstdint>

#if !defined(__CUDACC__) && !defined(__host__)
#define __host__
#endif
#if !defined(__CUDACC__) && !defined(__device__)
#define __device__
#endif

namespace gastar {

// Problem kinds compiled into the search kernel.
enum Kind : uint32_t { KIND_SLIDING3 = 0, KIND_SLIDING4 = 1, KIND_SLIDING5 = 2, KIND_GRID = 3, KIND_PLUGIN = 4 };
constexpr uint32_t kKindsAll = 0xf;
constexpr uint32_t kind_bit(uint32_t k) { return 1u << k; }

// Entries one stage buffer must hold: every popped entry of every warp-heap
// can stage all of its successors.  Dynamic shared memory of one block holds
// two stage buffers (one-block teams only) followed by the shared-memory heap
// nodes of every warp.
inline __host__ __device__ size_t stage_entries_per_buffer(uint32_t heaps, uint32_t ew, uint32_t maxn) {
    return (size_t)heaps * ew * maxn;
}

// Multi-block teams run their iterations without a team barrier.  Block b
// stages its successors of iteration i into region b of stage buffer
// i % kStageRing; after its expansion it publishes, behind one release fence,
// ready[b] = i + 1 and its part of cut i (heap minimum after the previous
// push, minimum of what it staged, goals, errors, counts).  Block c then
// pushes the region of block (c + i) % blocks once that block is ready.  Cut
// i is tested at iteration i + kCutLag, so no block runs more than kCutLag
// iterations ahead of another, and a stage buffer is always consumed before
// it is written again.
constexpr uint32_t kStageRing = 4;
constexpr uint32_t kCutLag = 2;
constexpr uint32_t kCuts = 16;  // cut slots in the ring (> 3 * kCutLag + 2)
// A block writes stage buffer i % kStageRing (and its ready words) in
// iteration i only after cut i - 1 - kCutLag is complete, i.e. after every
// block's push of iteration i - 2 - kCutLag: the buffer's previous use,
// iteration i - kStageRing, must be no later than that.
static_assert(kStageRing >= kCutLag + 2, "a stage buffer must be consumed before it is reused");

constexpr uint32_t kSlotsHost = 4;

// Plain engine: iteration from which a puzzle search with the automatic
// expansion width pops twice as many entries per warp-heap.
constexpr uint32_t kWideAfter = 64;

// Claim list: each warp reserves this many entries at a time; entries a warp
// reserved but did not use hold kTouchedHole.
constexpr uint32_t kTouchedChunk = 1024;
constexpr uint32_t kTouchedHole = 0xffffffffu;

// Warp-heap nodes below sn live in shared memory (node 0 in registers).
constexpr uint32_t kHeapSmemNodes = 7;      // default sn: nodes 1..6
// Dynamic shared memory above this needs the opt-in attribute: a block's
// static shared memory (the kernels' CtaShared, ~1.2 KB) counts against the
// default 48 KiB as well.
constexpr size_t kSmemNoOptIn = 44 * 1024;
constexpr uint32_t kHeapSmemNodesMax = 127;  // levels 0..6
// Global stage area of a multi-block team: kStageRing buffers, each one
// region of warps*ew*maxn entries per block; then one 64-bit ready word per
// region (kStageRing rows of `blocks` words): (iteration + 1) << 32 | the
// region's entry count, written when the region is complete.
inline __host__ __device__ size_t team_stage_bytes(uint32_t blocks, uint32_t warps, uint32_t ew, uint32_t maxn,
                                                   uint32_t entry_bytes) {
    const size_t entries = kStageRing * stage_entries_per_buffer(blocks * warps, ew, maxn);
    return ((entries * entry_bytes + (size_t)kStageRing * blocks * 8) + 15) & ~(size_t)15;
}

// Per-instance control block, written by the device.
struct alignas(16) InstCtl {
    uint32_t life;        // LIFE_FRESH / LIFE_RUNNING / LIFE_DONE
    uint32_t status;      // gastar_status of the finished search
    uint32_t best;        // best goal cost found (0xffffffff = none)
    uint32_t iterations;  // GA* iterations run so far
    uint32_t path_len;    // states on the rebuilt path
    uint32_t max_nodes;   // largest warp-heap size seen (32-entry nodes)
    uint64_t t_start;     // device globaltimer at the first iteration
    unsigned long long expansions, generated, pushes, stale, table_used;
    unsigned long long path_off;  // offset (64-bit words) of the path in the path arena
    uint64_t t_end;               // device globaltimer when the search finished
};

// Per-instance description, written by the host.
struct alignas(16) InstDesc {
    uint32_t kind, heuristic, moves, n;
    uint64_t start0, start1, goal0, goal1;  // packed keys (grid: cell index in start0/goal0)
    const uint8_t* weights;                 // grid: device pointer, w*h bytes
    uint32_t W, H, minw, f0;                // grid dims, minimum weight; f of the start
    unsigned long long* table;              // hash slots or dense value array
    uint64_t table_words;                   // 64-bit words in the table region
    uint64_t table_mask;                    // slots - 1 (hash tables)
    uint64_t table_limit;                   // claimed-slot limit before TABLE_FULL
    uint32_t max_probe, heaps;              // probe limit; warp-heaps of the instance
    void* heap_nodes;                       // heaps * (heap_cap + 1) * 32 entries
    uint32_t* heap_hdr;                     // heaps * 2 words
    uint32_t heap_cap, ew;                  // nodes per warp-heap; pops per heap per iteration
    uint64_t max_exp;                       // expansion budget (0 = none)
    uint64_t timeout_ns;                    // device deadline relative to t_start (0 = none)
    uint32_t max_iter, delta;               // iteration budget; pop window f <= fmin + delta (0 = off)
    InstCtl* ctl;
    // Reusable hash tables (plain engine): word offsets of the slots claimed by
    // the previous solve, cleared at the start of the next one instead of the
    // whole table.  touched == nullptr -> the whole table is cleared.
    uint32_t* touched;
    unsigned long long* touched_count;
    uint64_t touched_cap;
    uint32_t prev_slot_words;
    // 1: the list refers to this same table, which a whole-table clear may
    // replace when the list is long (batch partitions); 0: always the list
    // (the plain engine's buffer may have held a larger table before).
    uint32_t clear_either;
    uint64_t start_hi[2], goal_hi[2];  // key words 2..3 (generic plugin states)
    // Bucket front of the open list (bq_pages == 0 -> heaps only): per warp
    // bq_pages pages of 32 entries at bq_base, then the heaps' page links
    // (heaps * bq_pages words), then their free-page stacks (as many words),
    // then each heap's saved bucket state (kBucketStateWords words).
    void* bq_base;
    uint32_t bq_pages;
    // Widening (multi-block teams): from iteration wide_after on (0 = never)
    // each warp-heap pops up to ew_wide entries instead of ew; the stage
    // regions are sized for ew_wide.
    uint32_t ew_wide;
    uint32_t wide_after, pad2;
};

constexpr uint32_t kBucketStateWords = 128;

// Bytes of an instance's bucket area.
inline __host__ __device__ size_t bucket_area_bytes(uint32_t heaps, uint32_t pages, uint32_t entry_bytes) {
    return (size_t)heaps * pages * (32 * (size_t)entry_bytes + 8) + (size_t)heaps * kBucketStateWords * 4;
}

// Per-iteration state of a one-block team (shared memory); iteration t uses
// slot t % kSlots.
struct alignas(16) TeamSlot {
    unsigned long long minprio;   // min priority over the team's heaps after the push phase
    unsigned long long minstage;  // min priority of the entries staged in the pop/expand phase
    uint32_t count;               // entries staged in the pop/expand phase
    uint32_t best;                // goal costs found in the pop/expand phase
    uint32_t err;                 // first error raised in the iteration
    uint32_t pad;
};
constexpr uint32_t kSlots = 4;

// Control of a multi-block team (one instance on many blocks).
// One cut of a multi-block team: the state at the start of an iteration.
// Every block updates the minimum, the two counts and the arrival count of a
// slot with atomics in the same few hundred nanoseconds: each of them has its
// own 128-byte line, so those atomics queue at different L2 slices.
struct alignas(128) CutSlot {
    unsigned long long minprio;  // min priority over the team's heaps
    uint32_t best;               // goal costs found in the iteration before
    uint32_t lossy;              // entries were lost (table or heap full, cost range)
    uint32_t err;                // budget or timeout
    uint32_t pad0[27];
    unsigned long long claims;   // table slots the blocks claimed since their last cut
    uint32_t pad1[30];
    unsigned long long exps;     // expansions since the blocks' last cut
    uint32_t pad2[30];
    uint32_t count;              // blocks that published
    uint32_t pad3[31];
};
static_assert(sizeof(CutSlot) == 512, "one 128-byte line per contended word");

// The barrier counter only grows (barrier k of a team ends when it reaches
// (k+1) x blocks) and sits on its own 128-byte line, apart from the cut slots
// that every block updates with atomics.
struct alignas(128) TeamCtl {
    unsigned long long arrive;  // barrier arrivals since the team started
    uint32_t abort, inst;       // a block gave up; instance the team works on
    uint32_t pad[28];
    CutSlot cut[kCuts];
};
static_assert(offsetof(TeamCtl, cut) == 128, "the barrier counter and abort flag fill the first line");
inline void team_ctl_init(TeamCtl& t) {
    t.arrive = 0;
    t.abort = 0;
    t.inst = 0;
    for (auto& p : t.pad) p = 0;
    for (auto& c : t.cut) {
        c.minprio = ~0ull;
        c.claims = c.exps = 0;
        c.best = 0xffffffffu;
        c.lossy = c.err = c.count = 0;
    }
}

struct LaunchParams {
    const InstDesc* insts;
    uint32_t n_insts;
    uint32_t slice_iters;     // 0 = run each instance to completion
    const uint32_t* order;    // schedule order (nullptr = 0..n-1)
    uint32_t* next;           // work counter for single-block teams
    uint32_t team_ctas;       // 1 = one block per instance; >1 = all blocks on instance 0
    uint32_t heap_snodes;     // shared-memory heap nodes per warp + 1 (0 = kHeapSmemNodes)
    uint32_t buckets;         // 1 = blocks carry the bucket push scratch (some instance has buckets)
    uint32_t pad2;
    TeamCtl* team;            // multi-block team control (device)
    void* stage;              // multi-block stage buffer (device)
    uint64_t barrier_timeout_ns;
    // Heavy instances of a batch: blocks [0, heavy_teams * heavy_team) first
    // work in teams of heavy_team blocks on heavy_order[0..n_heavy), then join
    // the one-block loop.  Each team owns heavy_ctl[t] and a stage area of
    // heavy_stage_bytes at heavy_stage + t * heavy_stage_bytes.
    const uint32_t* heavy_order;
    uint32_t n_heavy, heavy_team, heavy_teams, pad1;
    uint32_t* heavy_next;
    TeamCtl* heavy_ctl;
    void* heavy_stage;
    uint64_t heavy_stage_bytes;
    const uint32_t* slices;   // per instance slot: iterations per slice (nullptr = slice_iters)
};

}  // namespace gastar
