// Device building blocks of the GA* engine: entries, warp sorting networks,
// the warp-cooperative batched binary heap and the duplicate-detection tables.
//
// Reference (michalborkowski96/cuda_a_star) counterparts:
//   HeapEntry / QueueValue ordering        heaps.h:14-23, a_star.h:55-66
//   HeapsDevice::extract/insert/remove     heaps.h:93-160   -> WarpHeap (below)
//   FancyHashmap mass insert + statuses    fancy_hashmap.h:32-167, 336-340
//                                          -> insert-or-min with CAS (below)
//   bitonic_sort network (global memory)   bitonic_sort.h:107-143
//                                          -> register/shuffle networks (below)
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gastar {

constexpr unsigned kFull = 0xffffffffu;
constexpr uint64_t kEmpty = ~0ull;      // empty table key / value
constexpr uint64_t kInfPrio = ~0ull;    // priority of a padding entry
constexpr uint32_t kInf = 0xffffffffu;
constexpr uint32_t kRootMove = 0xffu;   // parent move of the start state

// Device status codes; the numeric values are the gastar_status values of the C ABI.
enum : uint32_t {
    ST_OK = 0, ST_NO_PATH = 1, ST_BUDGET = 2, ST_TIMEOUT = 3, ST_HEAP_FULL = 4,
    ST_TABLE_FULL = 5, ST_PATH_CAP = 6, ST_BARRIER = 7, ST_BAD_INPUT = 8, ST_COST_RANGE = 13,
};
enum : uint32_t { LIFE_FRESH = 0, LIFE_RUNNING = 1, LIFE_DONE = 2 };

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t x) {
    // SplitMix64 output function (Steele, Lea, Flood 2014).
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

// Priority word: f in bits 63..32, (2^24-1 - g) in bits 31..8 and the move
// that produced the entry in bits 7..0, so that one unsigned comparison gives
// the reference's order "lower f first, equal f -> higher g first"
// (QueueValue::operator<, a_star.h:58-63) and a popped entry knows its parent
// move without a table lookup.  Costs are limited to kMaxG.
constexpr uint32_t kMaxG = 0xffffffu;
__host__ __device__ __forceinline__ uint64_t make_prio(uint32_t f, uint32_t g, uint32_t pm = 0xffu) {
    return (uint64_t(f) << 32) | (uint64_t(kMaxG - g) << 8) | (pm & 0xffu);
}
__host__ __device__ __forceinline__ uint32_t prio_f(uint64_t p) { return uint32_t(p >> 32); }
__host__ __device__ __forceinline__ uint32_t prio_g(uint64_t p) { return kMaxG - (uint32_t(p >> 8) & kMaxG); }
__host__ __device__ __forceinline__ uint32_t prio_pm(uint64_t p) { return uint32_t(p) & 0xffu; }

// Table value word: g in the high half, parent move in the low byte; one
// 64-bit atomicMin keeps the lowest g and, among equal g, the lowest move.
__host__ __device__ __forceinline__ uint64_t make_val(uint32_t g, uint32_t move) {
    return (uint64_t(g) << 32) | move;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---------------------------------------------------------------------------
// Heap entries: a priority word and KW 64-bit key words (KW = 1..4), padded to
// a multiple of 16 bytes: 16 B for 64-bit keys, 32 B for 128..192-bit keys,
// 48 B for 256-bit keys.
// ---------------------------------------------------------------------------
template <int KW> struct alignas(16) Entry {
    static constexpr int NK = KW + ((KW % 2 == 0) ? 1 : 0);  // key words incl. padding
    uint64_t prio;
    uint64_t k[NK];
};
template <int KW> __host__ __device__ constexpr int entry_vecs() { return (1 + Entry<KW>::NK) / 2; }

template <int KW> __device__ __forceinline__ Entry<KW> inf_entry() {
    Entry<KW> e;
    e.prio = kInfPrio;
#pragma unroll
    for (int j = 0; j < Entry<KW>::NK; ++j) e.k[j] = 0;
    return e;
}

template <int KW> __device__ __forceinline__ Entry<KW> shfl_idx(const Entry<KW>& e, int src) {
    Entry<KW> r;
    r.prio = __shfl_sync(kFull, e.prio, src);
#pragma unroll
    for (int j = 0; j < Entry<KW>::NK; ++j) r.k[j] = j < KW ? __shfl_sync(kFull, e.k[j], src) : 0;
    return r;
}

template <int KW> __device__ __forceinline__ Entry<KW> shfl_xor(const Entry<KW>& e, int m) {
    Entry<KW> r;
    r.prio = __shfl_xor_sync(kFull, e.prio, m);
#pragma unroll
    for (int j = 0; j < Entry<KW>::NK; ++j) r.k[j] = j < KW ? __shfl_xor_sync(kFull, e.k[j], m) : 0;
    return r;
}

template <int KW> __device__ __forceinline__ void set_word(Entry<KW>& e, int w, uint64_t v) {
    if (w == 0) e.prio = v;
    else e.k[w - 1] = v;
}
template <int KW> __device__ __forceinline__ uint64_t get_word(const Entry<KW>& e, int w) {
    return w == 0 ? e.prio : e.k[w - 1];
}

// L2-coherent loads/stores (heap nodes and stage buffers are handed between
// launches and, in multi-block teams, between blocks).
template <int KW> __device__ __forceinline__ Entry<KW> ld_entry(const Entry<KW>* p) {
    Entry<KW> e;
    const uint4* s = reinterpret_cast<const uint4*>(p);
#pragma unroll
    for (int v = 0; v < entry_vecs<KW>(); ++v) {
        const uint4 a = __ldcg(s + v);
        set_word(e, 2 * v, (uint64_t(a.y) << 32) | a.x);
        set_word(e, 2 * v + 1, (uint64_t(a.w) << 32) | a.z);
    }
    return e;
}
template <int KW> __device__ __forceinline__ void st_entry(Entry<KW>* p, const Entry<KW>& e) {
    uint4* d = reinterpret_cast<uint4*>(p);
#pragma unroll
    for (int v = 0; v < entry_vecs<KW>(); ++v) {
        const uint64_t a = get_word(e, 2 * v), b = get_word(e, 2 * v + 1);
        __stcg(d + v, make_uint4(uint32_t(a), uint32_t(a >> 32), uint32_t(b), uint32_t(b >> 32)));
    }
}

// Stage-buffer access: shared memory for one-block teams (plain generic
// accesses), global memory shared by the blocks of a multi-block team
// (L2-coherent accesses, since the buffer is refilled every iteration).
template <int KW> __device__ __forceinline__ Entry<KW> ld_stage(const Entry<KW>* p, bool global) {
    if (global) return ld_entry(p);
    Entry<KW> e;
    const uint4* s = reinterpret_cast<const uint4*>(p);
#pragma unroll
    for (int v = 0; v < entry_vecs<KW>(); ++v) {
        const uint4 a = s[v];
        set_word(e, 2 * v, (uint64_t(a.y) << 32) | a.x);
        set_word(e, 2 * v + 1, (uint64_t(a.w) << 32) | a.z);
    }
    return e;
}
template <int KW> __device__ __forceinline__ void st_stage(Entry<KW>* p, const Entry<KW>& e, bool global) {
    if (global) {
        st_entry(p, e);
        return;
    }
    uint4* d = reinterpret_cast<uint4*>(p);
#pragma unroll
    for (int v = 0; v < entry_vecs<KW>(); ++v) {
        const uint64_t a = get_word(e, 2 * v), b = get_word(e, 2 * v + 1);
        d[v] = make_uint4(uint32_t(a), uint32_t(a >> 32), uint32_t(b), uint32_t(b >> 32));
    }
}

// ---------------------------------------------------------------------------
// Warp sorting networks over one entry per lane (ascending by prio).
// Every compare-exchange decides from the same predicate in both lanes of a
// pair, so equal priorities never duplicate or drop an entry.
// ---------------------------------------------------------------------------
template <int KW> __device__ __forceinline__ Entry<KW> bitonic_clean(Entry<KW> x, int lane) {
#pragma unroll
    for (int j = 16; j > 0; j >>= 1) {
        Entry<KW> y = shfl_xor(x, j);
        bool lower = !(lane & j);
        bool sw = lower ? (y.prio < x.prio) : (x.prio < y.prio);
        if (sw) x = y;
    }
    return x;
}

template <int KW> __device__ __forceinline__ Entry<KW> sort32(Entry<KW> x, int lane) {
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            Entry<KW> y = shfl_xor(x, j);
            bool lower = !(lane & j);
            bool asc = (k == 32) || !(lane & k);
            bool sw = (lower == asc) ? (y.prio < x.prio) : (x.prio < y.prio);
            if (sw) x = y;
        }
    }
    return x;
}

// Merges two ascending 32-entry vectors: lo = 32 smallest, hi = 32 largest,
// both ascending.
template <int KW>
__device__ __forceinline__ void merge2(const Entry<KW>& a, const Entry<KW>& b, Entry<KW>& lo,
                                       Entry<KW>& hi, int lane) {
    Entry<KW> br = shfl_idx(b, 31 - lane);
    bool bl = br.prio < a.prio;
    lo = bl ? br : a;
    hi = bl ? a : br;
    lo = bitonic_clean(lo, lane);
    hi = bitonic_clean(hi, lane);
}

// Element idx (0..63) of the concatenation lo ++ hi; all lanes must call.
template <int KW>
__device__ __forceinline__ Entry<KW> pick(const Entry<KW>& lo, const Entry<KW>& hi, int idx) {
    Entry<KW> a = shfl_idx(lo, idx & 31);
    Entry<KW> b = shfl_idx(hi, idx & 31);
    return idx < 32 ? a : b;
}

// ---------------------------------------------------------------------------
// Warp-cooperative batched binary heap.
//
// One warp owns one heap.  A node holds 32 entries sorted ascending; the heap
// order is node-wise (every entry of a node <= every entry of its children),
// so the root holds the 32 best entries of the tree.  The root node and a
// partial buffer of < 32 entries live in registers (one entry per lane) for
// the lifetime of a launch, nodes 1..sn-1 in shared memory (the top levels;
// sn is chosen per launch from the shared memory left on the SM), the rest are 512-byte (or 1 KiB) blocks in global memory read and written with
// one coalesced access per lane.  Replaces the reference's one-thread-per-heap
// binary heaps with their key->slot index (heaps.h:93-177, device_hashmap.h):
// stale entries are dropped at pop time instead of being erased (lazy
// deletion).
// ---------------------------------------------------------------------------

template <int KW> struct WarpHeap {
    Entry<KW>* nodes;   // (cap + 1) * 32 entries; node `cap` stores the saved partial buffer
    Entry<KW>* snodes;  // shared memory: nodes 1..sn-1
    uint32_t* hdr;      // saved {N, pc}
    uint32_t cap;       // tree nodes available (>= sn)
    uint32_t sn;        // nodes below sn live in shared memory (node 0 in registers)
    uint32_t N;         // full nodes in the tree (warp-uniform)
    uint32_t pc;        // entries in the partial buffer (warp-uniform)
    uint32_t max_n;     // high-water mark of N
    Entry<KW> root;     // lane l: root[l] (valid iff N > 0)
    Entry<KW> part;     // lane l: partial[l] (valid iff l < pc), ascending
};

template <int KW>
__device__ __forceinline__ Entry<KW> ld_node(const WarpHeap<KW>& h, uint32_t idx, int lane) {
    if (idx < h.sn) return ld_stage(h.snodes + (size_t)(idx - 1) * 32 + lane, false);
    return ld_entry(h.nodes + (size_t)idx * 32 + lane);
}
template <int KW>
__device__ __forceinline__ void st_node(const WarpHeap<KW>& h, uint32_t idx, int lane, const Entry<KW>& e) {
    if (idx < h.sn) st_stage(h.snodes + (size_t)(idx - 1) * 32 + lane, e, false);
    else st_entry(h.nodes + (size_t)idx * 32 + lane, e);
}
// Priority of the largest entry of node idx (one read, broadcast to the warp).
template <int KW> __device__ __forceinline__ uint64_t node_max(const WarpHeap<KW>& h, uint32_t idx) {
    if (idx < h.sn) return *reinterpret_cast<const volatile uint64_t*>(&h.snodes[(size_t)(idx - 1) * 32 + 31].prio);
    return __ldcg(reinterpret_cast<const unsigned long long*>(&h.nodes[(size_t)idx * 32 + 31].prio));
}

// Starts bringing global node idx (each lane its own entry) into L2, so a
// dependent load of it later waits for L2 instead of DRAM.
template <int KW> __device__ __forceinline__ void prefetch_node(const WarpHeap<KW>& h, uint32_t idx, int lane) {
    if (idx >= h.sn && idx < h.N) {
        const Entry<KW>* a = h.nodes + (size_t)idx * 32 + lane;
        asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
    }
}

template <int KW> __device__ __forceinline__ void heap_init(WarpHeap<KW>& h) {
    h.N = 0;
    h.pc = 0;
    h.max_n = 0;
    h.root = inf_entry<KW>();
    h.part = inf_entry<KW>();
}

template <int KW> __device__ __forceinline__ void heap_restore(WarpHeap<KW>& h, int lane) {
    h.N = __ldcg(h.hdr);
    h.pc = __ldcg(h.hdr + 1);
    h.max_n = h.N;
    h.root = h.N ? ld_entry(h.nodes + lane) : inf_entry<KW>();
    h.part = (uint32_t)lane < h.pc ? ld_entry(h.nodes + (size_t)h.cap * 32 + lane) : inf_entry<KW>();
    for (uint32_t i = 1; i < h.N && i < h.sn; ++i)
        st_stage(h.snodes + (size_t)(i - 1) * 32 + lane, ld_entry(h.nodes + (size_t)i * 32 + lane), false);
    __syncwarp();
}

template <int KW> __device__ __forceinline__ void heap_save(const WarpHeap<KW>& h, int lane) {
    __syncwarp();
    if (h.N) st_entry(h.nodes + lane, h.root);
    for (uint32_t i = 1; i < h.N && i < h.sn; ++i)
        st_entry(h.nodes + (size_t)i * 32 + lane, ld_stage(h.snodes + (size_t)(i - 1) * 32 + lane, false));
    st_entry(h.nodes + (size_t)h.cap * 32 + lane, h.part);
    if (lane == 0) {
        __stcg(h.hdr, h.N);
        __stcg(h.hdr + 1, h.pc);
    }
}

template <int KW> __device__ __forceinline__ uint64_t heap_min(const WarpHeap<KW>& h) {
    uint64_t r = __shfl_sync(kFull, h.root.prio, 0);
    uint64_t p = __shfl_sync(kFull, h.part.prio, 0);
    r = h.N ? r : kInfPrio;
    p = h.pc ? p : kInfPrio;
    return r < p ? r : p;
}

// Restores the node order below the root after the root's content changed.
template <int KW> __device__ void heap_sift_down(WarpHeap<KW>& h, int lane) {
    Entry<KW> cur = h.root;
    uint32_t idx = 0;
    for (;;) {
        uint32_t l = 2 * idx + 1, r = l + 1;
        if (l >= h.N) break;
        Entry<KW> L = ld_node(h, l, lane);
        // The next level is a child of l or r: start all four on their way.
        prefetch_node(h, 2 * l + 1, lane);
        prefetch_node(h, 2 * l + 2, lane);
        prefetch_node(h, 2 * r + 1, lane);
        prefetch_node(h, 2 * r + 2, lane);
        uint64_t cmax = __shfl_sync(kFull, cur.prio, 31);
        uint64_t lmin = __shfl_sync(kFull, L.prio, 0);
        if (r >= h.N) {
            if (cmax > lmin) {
                Entry<KW> lo, hi;
                merge2(cur, L, lo, hi, lane);
                st_node(h, l, lane, hi);
                cur = lo;
            }
            break;
        }
        Entry<KW> R = ld_node(h, r, lane);
        uint64_t rmin = __shfl_sync(kFull, R.prio, 0);
        if (cmax <= (lmin < rmin ? lmin : rmin)) break;
        uint64_t lmax = __shfl_sync(kFull, L.prio, 31);
        uint64_t rmax = __shfl_sync(kFull, R.prio, 31);
        Entry<KW> A, B;
        merge2(L, R, A, B, lane);
        uint32_t big = lmax >= rmax ? l : r, small = big == l ? r : l;
        st_node(h, big, lane, B);  // B.max = max(lmax, rmax): big's subtree stays ordered
        Entry<KW> lo, hi;
        merge2(cur, A, lo, hi, lane);
        if (idx == 0) h.root = lo;
        else st_node(h, idx, lane, lo);
        cur = hi;
        idx = small;
    }
    if (idx == 0) h.root = cur;
    else st_node(h, idx, lane, cur);
    __syncwarp();
}

// Pops up to E (1..32) best entries whose priority is below `lim`; lane
// l < return value receives one.  Nothing changes when no entry qualifies.
template <int KW>
__device__ uint32_t heap_pop(WarpHeap<KW>& h, uint32_t E, uint64_t lim, Entry<KW>& out, int lane) {
    if (h.N == 0) {
        const uint32_t below = __popc(__ballot_sync(kFull, (uint32_t)lane < h.pc && h.part.prio < lim));
        const uint32_t c = E < below ? E : below;
        out = (uint32_t)lane < c ? h.part : inf_entry<KW>();
        Entry<KW> s = shfl_idx(h.part, (lane + (int)c) & 31);
        h.part = ((uint32_t)lane + c < h.pc) ? s : inf_entry<KW>();
        h.pc -= c;
        return c;
    }
    prefetch_node(h, h.N - 1, lane);  // the last node refills the root when the buffer runs short
    Entry<KW> lo, hi;
    merge2(h.root, h.part, lo, hi, lane);
    {
        const uint32_t below = __popc(__ballot_sync(kFull, lo.prio < lim));
        if (below < E) E = below;
        if (E == 0) {
            out = inf_entry<KW>();
            return 0;
        }
    }
    const uint32_t valid = 32 + h.pc, rest = valid - E;
    out = (uint32_t)lane < E ? lo : inf_entry<KW>();
    const int i1 = (int)E + lane, i2 = (int)E + 32 + lane;
    Entry<KW> r1 = pick(lo, hi, i1 & 63);
    Entry<KW> r2 = pick(lo, hi, i2 & 63);
    if ((uint32_t)i1 >= valid) r1 = inf_entry<KW>();
    if ((uint32_t)i2 >= valid) r2 = inf_entry<KW>();
    if (rest >= 32) {
        h.root = r1;
        h.part = r2;
        h.pc = rest - 32;
        heap_sift_down(h, lane);
    } else if (h.N == 1) {
        h.N = 0;
        h.root = inf_entry<KW>();
        h.part = r1;
        h.pc = rest;
    } else {
        Entry<KW> last = ld_node(h, h.N - 1, lane);
        h.N -= 1;
        Entry<KW> lo2, hi2;
        merge2(last, r1, lo2, hi2, lane);
        h.root = lo2;
        h.part = hi2;
        h.pc = rest;
        heap_sift_down(h, lane);
    }
    return E;
}

// Adds a full node top-down along the path to the new leaf: every node on the
// path keeps the 32 smallest of itself and the carried node.
template <int KW> __device__ bool heap_insert_node(WarpHeap<KW>& h, Entry<KW> F, int lane) {
    if (h.N == 0) {
        h.root = F;
        h.N = 1;
        if (h.max_n < 1) h.max_n = 1;
        return true;
    }
    if (h.N >= h.cap) return false;
    const uint32_t p = h.N + 1;
    const int levels = 31 - __clz(p);
    {
        uint64_t fmin = __shfl_sync(kFull, F.prio, 0);
        uint64_t rmax = __shfl_sync(kFull, h.root.prio, 31);
        if (fmin < rmax) {
            Entry<KW> lo, hi;
            merge2(h.root, F, lo, hi, lane);
            h.root = lo;
            F = hi;
        }
    }
    // The path is fixed by the new leaf's index: fetch the maximum of every
    // node on it in one parallel load (lane j <- depth j), so only the nodes
    // that need a merge cost a dependent access.
    uint64_t pmax = kInfPrio;
    if (lane >= 1 && lane < levels) pmax = node_max(h, (p >> (levels - lane)) - 1);
    for (int b = levels - 1; b >= 1; --b) prefetch_node(h, (p >> b) - 1, lane);  // the nodes themselves
    for (int b = levels - 1; b >= 1; --b) {
        const uint32_t idx = (p >> b) - 1;
        uint64_t fmin = __shfl_sync(kFull, F.prio, 0);
        if (fmin < __shfl_sync(kFull, pmax, levels - b)) {
            Entry<KW> M = ld_node(h, idx, lane);
            Entry<KW> lo, hi;
            merge2(M, F, lo, hi, lane);
            st_node(h, idx, lane, lo);
            F = hi;
        }
    }
    st_node(h, h.N, lane, F);
    __syncwarp();
    h.N += 1;
    if (h.N > h.max_n) h.max_n = h.N;
    return true;
}

// Pushes up to 32 entries (lanes >= m must hold padding entries).
template <int KW>
__device__ bool heap_push(WarpHeap<KW>& h, Entry<KW> x, uint32_t m, int lane) {
    if (m == 0) return true;
    x = sort32(x, lane);
    Entry<KW> lo, hi;
    merge2(h.part, x, lo, hi, lane);
    const uint32_t tot = h.pc + m;
    if (tot < 32) {
        h.part = lo;
        h.pc = tot;
        return true;
    }
    // The largest 32 form a new node; the smallest stay in the partial buffer,
    // where the next pop sees them first.
    const uint32_t off = tot - 32;
    Entry<KW> node = pick(lo, hi, (int)off + lane);
    h.part = (uint32_t)lane < off ? lo : inf_entry<KW>();
    h.pc = off;
    return heap_insert_node(h, node, lane);
}

// ---------------------------------------------------------------------------
// Bucket front of a warp's open list.
//
// Entries whose f lies in the window [lo, lo + 32) go to one of 32 buckets
// (bucket = f mod 32; lane b keeps bucket b's state), each a stack of 32-entry
// pages in global memory.  Every other entry -- and every entry once the
// pages run out -- goes to the warp-heap.  A pop takes from whichever holds
// the lower f; the buckets are exact in f and last-in first-out within one f,
// which favours the deepest entries among equal f as the heap's g tie-break
// does, so the open list's minimum stays exact.  A push is a few shuffles and
// stores, a pop one coalesced page load, where the heap merges 32-entry nodes
// level by level (two 64-entry merges of ~44 shuffles each per level).
// Pages come from a cache of free page ids held in registers (lane l < fc
// holds one), then from never-used pages (bump), then from a stack in global
// memory of pages freed while the cache was full.
// ---------------------------------------------------------------------------
constexpr uint32_t kNoPage = 0xffffffffu;

template <int KW> struct Buckets {
    Entry<KW>* pages;  // P pages of 32 entries (global memory)
    uint32_t* link;    // the page below each page in its bucket's stack (global memory)
    uint32_t* fstack;  // pages freed while the register cache was full (global memory)
    uint32_t* upd;     // per-bucket scratch of a push (64 words, shared memory)
    uint32_t* state;   // saved state of a suspended search (global memory)
    uint32_t P;        // pages (0 = buckets off)
    uint32_t bump;     // pages >= bump were never used (warp-uniform)
    uint32_t nfs;      // entries on fstack (warp-uniform)
    uint32_t fc;       // free page ids cached in registers (warp-uniform)
    uint32_t cache;    // lane l < fc: a free page id
    uint32_t lo;       // window start (warp-uniform)
    uint32_t head;     // lane b: top page of bucket b (kNoPage = empty)
    uint32_t hcnt;     // lane b: entries in that page (the pages below are full)
};

template <int KW> __device__ __forceinline__ void bq_init(Buckets<KW>& q, int) {
    q.bump = 0;
    q.nfs = 0;
    q.fc = 0;
    q.cache = kNoPage;
    q.lo = 0;
    q.head = kNoPage;
    q.hcnt = 0;
}

// f of the lowest non-empty bucket, or kInf.
template <int KW> __device__ __forceinline__ uint32_t bq_min_f(const Buckets<KW>& q) {
    const uint32_t mask = __ballot_sync(kFull, q.head != kNoPage);
    if (!mask) return kInf;
    const uint32_t s = q.lo & 31u;
    const uint32_t rot = s ? (mask >> s) | (mask << (32 - s)) : mask;
    return q.lo + (uint32_t)(__ffs(rot) - 1);
}

template <int KW> __device__ __forceinline__ uint64_t open_min(const WarpHeap<KW>& h, const Buckets<KW>& q) {
    const uint64_t hm = heap_min(h);
    if (!q.P) return hm;
    const uint32_t bf = bq_min_f(q);
    const uint64_t bp = bf == kInf ? kInfPrio : ((uint64_t)bf << 32);
    return hm < bp ? hm : bp;
}

// Returns a freed page to the cache, or to the global stack when it is full.
template <int KW> __device__ __forceinline__ void bq_free(Buckets<KW>& q, uint32_t page, int lane) {
    if (q.fc < 32) {
        if ((uint32_t)lane == q.fc) q.cache = page;
        q.fc += 1;
    } else {
        if (lane == 0) __stcg(q.fstack + q.nfs, page);
        q.nfs += 1;
    }
}

// Adds x (lanes < m valid; lanes >= m hold inf entries).  Returns false when
// the heap is full (entries were lost).
template <int KW>
__device__ bool open_push(WarpHeap<KW>& h, Buckets<KW>& q, Entry<KW> x, uint32_t m, int lane) {
    if (m == 0) return true;
    const bool valid = (uint32_t)lane < m;
    bool placed = false;
    if (q.P) {
        const uint32_t f = prio_f(x.prio);
        if (!__any_sync(kFull, q.head != kNoPage)) {  // empty: the window starts at the least f
            uint32_t mf = valid ? f : kInf;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const uint32_t t = __shfl_xor_sync(kFull, mf, o);
                mf = t < mf ? t : mf;
            }
            q.lo = mf;
        }
        const bool inwin = valid && f >= q.lo && f - q.lo < 32u;
        const uint32_t b = f & 31u;
        const uint32_t lt = (1u << lane) - 1u;
        const uint32_t grp = __match_any_sync(kFull, inwin ? b : 32u + (uint32_t)lane);
        const uint32_t r = __popc(grp & lt), n = __popc(grp);
        const uint32_t hd = __shfl_sync(kFull, q.head, (int)b), hc = __shfl_sync(kFull, q.hcnt, (int)b);
        const bool leader = inwin && r == 0;
        const uint32_t room = hd == kNoPage ? 0u : 32u - hc;
        const bool need = inwin && n > room;
        // One new page per overflowing bucket: cached ids first, then
        // never-used pages, then the global stack.
        const uint32_t nmask = __ballot_sync(kFull, leader && need);
        const uint32_t want = __popc(nmask);
        const uint32_t fresh = q.P - q.bump, avail = q.fc + fresh + q.nfs;
        uint32_t page = kNoPage;
        {
            const uint32_t idx = __popc(nmask & lt);
            const uint32_t cached = __shfl_sync(kFull, q.cache, (int)((q.fc - 1 - idx) & 31u));
            if (leader && need && idx < avail) {
                if (idx < q.fc) page = cached;
                else if (idx < q.fc + fresh) page = q.bump + (idx - q.fc);
                else page = __ldcg(q.fstack + q.nfs - 1 - (idx - q.fc - fresh));
            }
        }
        {
            uint32_t take = want < avail ? want : avail;
            const uint32_t from_cache = take < q.fc ? take : q.fc;
            q.fc -= from_cache;
            take -= from_cache;
            const uint32_t from_bump = take < fresh ? take : fresh;
            q.bump += from_bump;
            q.nfs -= take - from_bump;
        }
        page = __shfl_sync(kFull, page, __ffs(grp) - 1);
        if (inwin) {
            if (r < room) {
                st_entry(q.pages + (size_t)hd * 32 + hc + r, x);
                placed = true;
            } else if (page != kNoPage) {
                st_entry(q.pages + (size_t)page * 32 + (r - room), x);
                placed = true;
            }
        }
        if (leader) {
            uint32_t nh = hd, nc = hc;
            if (n <= room) {
                nc = hc + n;
            } else {
                if (hd != kNoPage) nc = 32;
                if (page != kNoPage) {
                    __stcg(q.link + page, hd);
                    nh = page;
                    nc = n - room;
                }
            }
            q.upd[2 * b] = nh;
            q.upd[2 * b + 1] = nc;
        }
        const uint32_t umask = __reduce_or_sync(kFull, leader ? (1u << b) : 0u);
        __syncwarp();
        if ((umask >> lane) & 1u) {
            q.head = q.upd[2 * lane];
            q.hcnt = q.upd[2 * lane + 1];
        }
        __syncwarp();
    }
    const bool rest = valid && !placed;
    const uint32_t rm = __ballot_sync(kFull, rest);
    if (!rm) return true;
    return heap_push(h, rest ? x : inf_entry<KW>(), (uint32_t)__popc(rm), lane);
}

// Pops up to E (1..32) entries with priority below `lim` (a multiple of 2^32
// or kInfPrio); lane l < return value receives one.
template <int KW>
__device__ uint32_t open_pop(WarpHeap<KW>& h, Buckets<KW>& q, uint32_t E, uint64_t lim, Entry<KW>& out,
                             int lane) {
    if (!q.P) return heap_pop(h, E, lim, out, lane);
    out = inf_entry<KW>();
    uint32_t taken = 0;
    for (int round = 0; round < 4 && taken < E; ++round) {
        const uint32_t bf = bq_min_f(q);
        const uint64_t hm = heap_min(h);
        const uint64_t bp = bf == kInf ? kInfPrio : ((uint64_t)bf << 32);
        if ((hm < bp ? hm : bp) >= lim) break;
        const uint32_t i = (uint32_t)lane - taken;  // this lane's index among the new ones
        if (hm < bp) {  // the heap holds lower f: take its entries below the buckets' f
            Entry<KW> e;
            const uint32_t c = heap_pop(h, E - taken, bp < lim ? bp : lim, e, lane);
            const Entry<KW> sh = shfl_idx(e, (lane - (int)taken) & 31);
            if ((uint32_t)lane >= taken && i < c) out = sh;
            taken += c;
            if (c == 0) break;
        } else {
            const int bl = (int)(bf & 31u);
            const uint32_t hd = __shfl_sync(kFull, q.head, bl), hc = __shfl_sync(kFull, q.hcnt, bl);
            const uint32_t k = E - taken < hc ? E - taken : hc;
            // The page's entries and, when it empties, its link load together.
            const uint32_t nx = hc == k ? __ldcg(q.link + hd) : kNoPage;
            if ((uint32_t)lane >= taken && i < k) out = ld_entry(q.pages + (size_t)hd * 32 + (hc - k + i));
            if (hc == k) {  // the page is empty: the next one comes up, this one is free
                if (lane == bl) {
                    q.head = nx;
                    q.hcnt = nx == kNoPage ? 0u : 32u;
                }
                bq_free(q, hd, lane);
            } else if (lane == bl) {
                q.hcnt = hc - k;
            }
            taken += k;
        }
    }
    const uint32_t bf = bq_min_f(q);
    if (bf != kInf) q.lo = bf;  // the window follows the lowest non-empty bucket
    return taken;
}

// The bucket state of a suspended search stays beside its pages: lane l
// saves its bucket's head page and count and its cached free page; lane 0
// the window start, the never-used and free-stack counts and the cache size.
template <int KW> __device__ __forceinline__ void bq_save(const Buckets<KW>& q, int lane) {
    if (!q.P) return;
    __stcg(q.state + lane, q.head);
    __stcg(q.state + 32 + lane, q.hcnt);
    __stcg(q.state + 64 + lane, q.cache);
    if (lane == 0) {
        __stcg(q.state + 96, q.lo);
        __stcg(q.state + 97, q.bump);
        __stcg(q.state + 98, q.nfs);
        __stcg(q.state + 99, q.fc);
    }
}
template <int KW> __device__ __forceinline__ void bq_restore(Buckets<KW>& q, int lane) {
    if (!q.P) return;
    q.head = __ldcg(q.state + lane);
    q.hcnt = __ldcg(q.state + 32 + lane);
    q.cache = __ldcg(q.state + 64 + lane);
    q.lo = __ldcg(q.state + 96);
    q.bump = __ldcg(q.state + 97);
    q.nfs = __ldcg(q.state + 98);
    q.fc = __ldcg(q.state + 99);
}

// ---------------------------------------------------------------------------
// Duplicate-detection tables.  insert-or-min returns the previous value word;
// the caller keeps a successor iff its g is strictly below the old g.  This is
// the reference's NEW -> INSERTED / UPDATED / REJECTED classification
// (fancy_hashmap.h:32-81, 155-167) as one atomic per successor.
// ---------------------------------------------------------------------------

// Claim protocol shared by the tables.  claim_first / claim_probe return
//   -1 full, 2 home slot taken by another key (claim_probe walks on),
//   0 found / 1 claimed, with `old` the value word before this update (done),
//   4 found / 5 claimed, with the value still to be lowered by min_at.
constexpr int kClNeedMin = 4;

__device__ __forceinline__ void cas128(unsigned long long* addr, uint64_t c0, uint64_t c1,
                                       uint64_t n0, uint64_t n1, uint64_t& o0, uint64_t& o1) {
    asm volatile(
        "{\n\t.reg .b128 cmp, swp, dst;\n\t"
        "mov.b128 cmp, {%2, %3};\n\t"
        "mov.b128 swp, {%4, %5};\n\t"
        "atom.global.cas.b128 dst, [%6], cmp, swp;\n\t"
        "mov.b128 {%0, %1}, dst;\n\t}"
        : "=l"(o0), "=l"(o1)
        : "l"(c0), "l"(c1), "l"(n0), "l"(n1), "l"(addr)
        : "memory");
}

// 64-bit keys: slot = {key, value}, 16 bytes; linear probing.  Every atomic
// on a slot is one 16-byte compare-and-swap of the pair: a new key is claimed
// with its value in one round trip, a known key costs none more unless its
// value drops.
struct HashTab64 {
    unsigned long long* s;
    uint64_t mask;
    uint32_t max_probe;
};

__device__ __forceinline__ int tab_claim_at(const HashTab64& t, uint64_t i, uint64_t key, uint64_t val,
                                            uint64_t& old) {
    uint64_t o0, o1;
    cas128(t.s + 2 * i, kEmpty, kEmpty, key, val, o0, o1);
    if (o0 == kEmpty && o1 == kEmpty) {
        old = kEmpty;
        return 1;
    }
    if (o0 != key) return 2;
    old = o1;
    return o1 > val ? kClNeedMin : 0;
}
__device__ __forceinline__ int tab_claim_first(const HashTab64& t, uint64_t key, uint64_t val, uint64_t& slot,
                                               uint64_t& old) {
    const uint64_t i = mix64(key) & t.mask;
    slot = 2 * i;
    return tab_claim_at(t, i, key, val, old);
}
__device__ __forceinline__ int tab_claim_probe(const HashTab64& t, uint64_t key, uint64_t val, uint64_t& slot,
                                               uint64_t& old) {
    uint64_t i = slot / 2;
    for (uint32_t p = 1; p < t.max_probe; ++p) {
        i = (i + 1) & t.mask;
        const int r = tab_claim_at(t, i, key, val, old);
        if (r != 2) {
            slot = 2 * i;
            return r;
        }
    }
    return -1;
}
// Lowers the value of a found key to `val` unless it is already <= val;
// `seen` is the value the claim read.  Returns the value before the update.
// Values only fall, so every failed exchange is followed by a strictly lower
// value; the retry bound is far beyond the number of concurrent updaters.
__device__ __forceinline__ uint64_t tab_min_at(const HashTab64& t, uint64_t slot, uint64_t key, uint64_t val,
                                               uint64_t seen) {
    uint64_t cur = seen;
    for (uint32_t r = 0; cur > val && r < 4096; ++r) {
        uint64_t o0, o1;
        cas128(t.s + slot, key, cur, key, val, o0, o1);
        if (o1 == cur) break;
        cur = o1;
    }
    return cur;
}
// Returns 1 when the key was newly claimed, 0 when found, -1 when full.
__device__ __forceinline__ int tab_insert(const HashTab64& t, uint64_t key, uint64_t val, uint64_t& old,
                                          uint64_t& slot) {
    int r = tab_claim_first(t, key, val, slot, old);
    if (r == 2) r = tab_claim_probe(t, key, val, slot, old);
    if (r == kClNeedMin) {
        old = tab_min_at(t, slot, key, val, old);
        r = 0;
    }
    return r;
}

// Two-step lookup: look_begin issues the home-slot load, look_end resolves
// it (probing on when the home slot holds another key), so the load can be in
// flight while other memory work is issued.
struct Look64 {
    unsigned long long k, v;
};
__device__ __forceinline__ Look64 tab_look_begin(const HashTab64& t, uint64_t key) {
    const uint64_t i = mix64(key) & t.mask;
    const ulonglong2 kv = __ldcg(reinterpret_cast<const ulonglong2*>(t.s + 2 * i));
    return Look64{kv.x, kv.y};
}

__device__ __forceinline__ uint64_t tab_get(const HashTab64& t, uint64_t key) {
    uint64_t i = mix64(key) & t.mask;
    for (uint32_t p = 0; p < t.max_probe; ++p) {
        // Key and value in one 16-byte load (they are written together).
        const ulonglong2 kv = __ldcg(reinterpret_cast<const ulonglong2*>(t.s + 2 * i));
        if (kv.x == key) return kv.y;
        if (kv.x == kEmpty) return kEmpty;
        i = (i + 1) & t.mask;
    }
    return kEmpty;
}

// 128-bit keys: slot = {k0, k1, value, pad}, 32 bytes (one sector).  The key
// is claimed with a 16-byte compare-and-swap; reads of the key pair also go
// through the 16-byte atomic so a half-written pair is never observed.
struct HashTab128 {
    unsigned long long* s;
    uint64_t mask;
    uint32_t max_probe;
};

__device__ __forceinline__ uint64_t hash128(uint64_t k0, uint64_t k1) {
    return mix64(k0 ^ mix64(k1 + 0x9e3779b97f4a7c15ull));
}

__device__ __forceinline__ int tab_insert(const HashTab128& t, uint64_t k0, uint64_t k1,
                                          uint64_t val, uint64_t& old, uint64_t& slot) {
    uint64_t i = hash128(k0, k1) & t.mask;
    for (uint32_t p = 0; p < t.max_probe; ++p) {
        unsigned long long* ks = t.s + 4 * i;
        uint64_t o0, o1;
        cas128(ks, kEmpty, kEmpty, k0, k1, o0, o1);
        int claimed = (o0 == kEmpty && o1 == kEmpty);
        if (claimed || (o0 == k0 && o1 == k1)) {
            old = atomicMin(ks + 2, val);
            slot = 4 * i;
            return claimed;
        }
        i = (i + 1) & t.mask;
    }
    return -1;
}

__device__ __forceinline__ uint64_t tab_get(const HashTab128& t, uint64_t k0, uint64_t k1) {
    uint64_t i = hash128(k0, k1) & t.mask;
    for (uint32_t p = 0; p < t.max_probe; ++p) {
        unsigned long long* ks = t.s + 4 * i;
        uint64_t o0, o1;
        cas128(ks, kEmpty, kEmpty, kEmpty, kEmpty, o0, o1);  // atomic 16-byte read
        if (o0 == k0 && o1 == k1) return __ldcg(ks + 2);
        if (o0 == kEmpty && o1 == kEmpty) return kEmpty;
        i = (i + 1) & t.mask;
    }
    return kEmpty;
}

// Dense table for grids: the cell index is the slot (a perfect hash).
struct DenseTab {
    unsigned long long* v;
};

// 128-bit keys: the key pair is claimed with a 16-byte compare-and-swap, the
// value word beside it is lowered with atomicMin.
__device__ __forceinline__ int tab_claim_first(const HashTab128& t, uint64_t k0, uint64_t k1, uint64_t& slot) {
    const uint64_t i = hash128(k0, k1) & t.mask;
    slot = 4 * i;
    uint64_t o0, o1;
    cas128(t.s + 4 * i, kEmpty, kEmpty, k0, k1, o0, o1);
    if (o0 == kEmpty && o1 == kEmpty) return kClNeedMin | 1;
    return (o0 == k0 && o1 == k1) ? kClNeedMin : 2;
}
__device__ __forceinline__ int tab_claim_probe(const HashTab128& t, uint64_t k0, uint64_t k1, uint64_t& slot) {
    uint64_t i = slot / 4;
    for (uint32_t p = 1; p < t.max_probe; ++p) {
        i = (i + 1) & t.mask;
        uint64_t o0, o1;
        cas128(t.s + 4 * i, kEmpty, kEmpty, k0, k1, o0, o1);
        const int claimed = (o0 == kEmpty && o1 == kEmpty);
        if (claimed || (o0 == k0 && o1 == k1)) {
            slot = 4 * i;
            return kClNeedMin | claimed;
        }
    }
    return -1;
}
__device__ __forceinline__ uint64_t tab_min_at(const HashTab128& t, uint64_t slot, uint64_t val) {
    return atomicMin(t.s + slot + 2, val);
}

}  // namespace gastar
