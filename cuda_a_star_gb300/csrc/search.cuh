// The GA* search: problem domains and the persistent search kernel.
//
// One "team" of thread blocks works on one instance; each warp of the team
// owns one open list (a warp-heap, optionally behind a bucket front).  An
// iteration is
//   pop    : every warp pops up to `ew` best entries (one per lane), drops
//            stale ones (table g lower than the entry's g) and goal states;
//   expand : every lane generates the successors of its entry, computes g and
//            an incrementally updated h, and does one insert-or-min on the
//            duplicate-detection table per successor; improved successors go
//            to the block's stage area;
//   push   : one-block teams deal their stage chunks round-robin (rotating
//            offset) to their warps after a block barrier; in a multi-block
//            team block c pushes the stage region of block (c + i) mod blocks
//            once that block has flagged it ready (no team barrier);
//   check  : the search ends when the best goal cost is <= min f over all
//            open entries -- over the block's slots (one-block teams) or over
//            the cut every block publishes with its stage region, one
//            hand-off per iteration (multi-block teams, tested kCutLag
//            iterations later).
// This is the reference's iteration (a_star.h:247-264: extract_nodes, three
// bitonic sorts, mark_duplicates, insert_unique_data, remove_updated_elements,
// insert_nodes_into_queues, two host reductions) as one device-resident loop
// with no host round trip.
#pragma once

#include <type_traits>

#include "device_common.cuh"
#include "engine_types.h"

namespace gastar {

// ---------------------------------------------------------------------------
// Sliding puzzle, n x n.  Keys pack the tile of cell i in bits [B*i, B*i+B)
// (B = 4 for n <= 4 in a uint64, B = 5 for n = 5 in 128 bits).  Moves follow
// the reference's neighbour_generator (a_star_sliding_puzzle.h:84-123):
// move 0/1/2/3 moves the blank row+1 / row-1 / col+1 / col-1, cost 1.
// ---------------------------------------------------------------------------
template <int N> struct SlidingDom {
    static constexpr int KW = N <= 4 ? 1 : 2;
    static constexpr int MAXN = 4;
    static constexpr int B = N <= 4 ? 4 : 5;
    static constexpr int C = N * N;
    using KeyT = std::conditional_t<KW == 1, uint64_t, unsigned __int128>;
    using Tab = std::conditional_t<KW == 1, HashTab64, HashTab128>;
    using Pre = int;  // blank cell

    struct Ctx {
        KeyT goal, start;
        uint32_t ref_h, ref_moves;
        uint8_t md[C][C];  // md[t][p]: Manhattan distance of tile t placed at cell p
    };

    static __device__ __forceinline__ uint32_t field(KeyT k, int i) {
        return uint32_t(k >> (B * i)) & ((1u << B) - 1);
    }
    static __device__ __forceinline__ KeyT key_of(const Entry<KW>& e) {
        if constexpr (KW == 1) return e.k[0];
        else return (KeyT(e.k[1]) << 64) | KeyT(e.k[0]);
    }
    static __device__ __forceinline__ void set_key(Entry<KW>& e, KeyT k) {
        e.k[0] = uint64_t(k);
        if constexpr (KW == 2) e.k[1] = uint64_t(k >> 64);
    }
    static __device__ __forceinline__ KeyT desc_key(uint64_t lo, uint64_t hi) {
        if constexpr (KW == 1) return lo;
        else return (KeyT(hi) << 64) | KeyT(lo);
    }

    // Cell of the blank: the unique all-zero field, found with an AND-fold of
    // the complemented key.
    static __device__ __forceinline__ int blank_of(KeyT k) {
        KeyT y = ~k;
        KeyT z = y & (y >> 1);
        z = z & (z >> 2);
        if constexpr (B == 5) z = z & (y >> 4);
        KeyT mask = 0;
#pragma unroll
        for (int i = 0; i < C; ++i) mask |= KeyT(1) << (B * i);
        z &= mask;
        if constexpr (KW == 1) {
            return (__ffsll((long long)z) - 1) / B;
        } else {
            uint64_t lo = uint64_t(z), hi = uint64_t(z >> 64);
            int bit = lo ? __ffsll((long long)lo) - 1 : 64 + __ffsll((long long)hi) - 1;
            return bit / B;
        }
    }

    static __device__ void load(Ctx& c, const InstDesc& d) {
        const KeyT goal = desc_key(d.goal0, d.goal1);
        for (int i = threadIdx.x; i < C * C; i += blockDim.x) {
            const int t = i / C, p = i % C;
            int gp = 0;
            for (int q = 0; q < C; ++q)
                if ((int)field(goal, q) == t) gp = q;
            int v = abs(gp / N - p / N) + abs(gp % N - p % N);
            c.md[t][p] = d.heuristic == 2 ? 0 : (uint8_t)v;
        }
        if (threadIdx.x == 0) {
            c.goal = goal;
            c.start = desc_key(d.start0, d.start1);
            c.ref_h = d.heuristic == 1;
            c.ref_moves = d.moves == 1;
        }
        __syncthreads();
    }

    static __device__ __forceinline__ Tab make_tab(const InstDesc& d) {
        Tab t;
        t.s = d.table;
        t.mask = d.table_mask;
        t.max_probe = d.max_probe;
        return t;
    }
    static __device__ __forceinline__ uint64_t get(const Tab& t, KeyT k) {
        if constexpr (KW == 1) return tab_get(t, k);
        else return tab_get(t, uint64_t(k), uint64_t(k >> 64));
    }
    static __device__ __forceinline__ uint32_t start_f(const Ctx&, const InstDesc& d) { return d.f0; }
    // Parents are recorded by move code; the root's code is kRootMove.
    static constexpr uint32_t kRootCode = kRootMove;
    static constexpr bool kParentBySlot = false;
    struct Look {
        uint64_t k, v;
    };
    static __device__ __forceinline__ Look look_begin(const Tab& t, KeyT k) {
        if constexpr (KW == 1) {
            const Look64 l = tab_look_begin(t, k);
            return Look{l.k, l.v};
        } else {
            return Look{0, 0};
        }
    }
    static __device__ __forceinline__ uint64_t look_end(const Tab& t, KeyT k, const Look& l) {
        if constexpr (KW == 1) {
            if (l.k == k) return l.v;
            if (l.k == kEmpty) return kEmpty;
        }
        return get(t, k);
    }
    static __device__ __forceinline__ uint64_t get_self(const Tab& t, KeyT k, uint32_t&) { return get(t, k); }
    static __device__ __forceinline__ uint32_t code(int m, uint32_t) { return (uint32_t)m; }
    static __device__ __forceinline__ int insert(const Tab& t, KeyT k, uint64_t v, uint64_t& old,
                                                 uint64_t& slot) {
        if constexpr (KW == 1) return tab_insert(t, k, v, old, slot);
        else return tab_insert(t, uint64_t(k), uint64_t(k >> 64), v, old, slot);
    }
    static constexpr bool kDense = false;
    static __device__ __forceinline__ int claim_first(const Tab& t, KeyT k, uint64_t v, uint64_t& slot,
                                                      uint64_t& old) {
        if constexpr (KW == 1) return tab_claim_first(t, k, v, slot, old);
        else return tab_claim_first(t, uint64_t(k), uint64_t(k >> 64), slot);
    }
    static __device__ __forceinline__ int claim_probe(const Tab& t, KeyT k, uint64_t v, uint64_t& slot,
                                                      uint64_t& old) {
        if constexpr (KW == 1) return tab_claim_probe(t, k, v, slot, old);
        else return tab_claim_probe(t, uint64_t(k), uint64_t(k >> 64), slot);
    }
    static __device__ __forceinline__ uint64_t min_at(const Tab& t, uint64_t slot, KeyT k, uint64_t v,
                                                      uint64_t seen) {
        if constexpr (KW == 1) return tab_min_at(t, slot, k, v, seen);
        else return tab_min_at(t, slot, v);
    }
    static __device__ __forceinline__ bool is_goal(const Ctx& c, KeyT k) { return k == c.goal; }
    static __device__ __forceinline__ bool is_start(const Ctx& c, KeyT k) { return k == c.start; }
    static __device__ __forceinline__ Pre prepare(const Ctx&, KeyT k) { return blank_of(k); }

    static __device__ __forceinline__ bool succ(const Ctx& c, KeyT k, Pre p, int m, uint32_t pm,
                                                uint32_t g, uint32_t h, KeyT& nk, uint32_t& ng,
                                                uint32_t& nh) {
        if ((uint32_t)(m ^ 1) == pm) return false;  // straight back to the parent
        const int r = p / N, col = p % N;
        int q;
        if (m == 0) {
            if (r >= N - 1) return false;
            q = p + N;
        } else if (m == 1) {
            if (c.ref_moves || r == 0) return false;
            q = p - N;
        } else if (m == 2) {
            if (col >= N - 1) return false;
            q = p + 1;
        } else {
            if (c.ref_moves || col == 0) return false;
            q = p - 1;
        }
        const uint32_t t = field(k, q);
        nk = (k & ~(KeyT((1u << B) - 1) << (B * q))) | (KeyT(t) << (B * p));
        nh = h + c.md[t][p] - c.md[t][q];
        if (c.ref_h) nh = nh + c.md[0][q] - c.md[0][p];
        ng = g + 1;
        return true;
    }

    // Parent of k when k was reached with move m: the blank moves back.
    static __device__ __forceinline__ KeyT parent(const Ctx&, const Tab&, KeyT k, uint32_t m) {
        const int p = blank_of(k);
        const int q = (m == 0) ? p - N : (m == 1) ? p + N : (m == 2) ? p - 1 : p + 1;
        const uint32_t t = field(k, q);
        return (k & ~(KeyT((1u << B) - 1) << (B * q))) | (KeyT(t) << (B * p));
    }
};

// ---------------------------------------------------------------------------
// Weighted grid, 8-connected (a_star_pathfinding.h:147-209).  Key = cell index
// y*W + x.  Move m shifts (x, y) by (DX[m], DY[m]); entering a cell costs its
// weight; weight 0 is impassable.  The duplicate-detection table is a dense
// value array indexed by cell.
// ---------------------------------------------------------------------------
struct GridDom {
    static constexpr int KW = 1;
    static constexpr int MAXN = 8;
    using KeyT = uint64_t;
    using Tab = DenseTab;
    struct Pre {
        int x, y;
        uint64_t wts;  // byte m: weight of the cell move m enters (0 = obstacle or off the board)
    };

    struct Ctx {
        const uint8_t* w;
        uint32_t W, H, goal, start, gx, gy, minw, href;
    };

    static __device__ __forceinline__ int dx(int m) { return (m == 0 || m == 4 || m == 5) ? 1 : (m == 1 || m == 6 || m == 7) ? -1 : 0; }
    static __device__ __forceinline__ int dy(int m) { return (m == 2 || m == 4 || m == 6) ? 1 : (m == 3 || m == 5 || m == 7) ? -1 : 0; }
    static __device__ __forceinline__ uint32_t inv(uint32_t m) { return m < 4 ? (m ^ 1) : 11 - m; }

    static __device__ __forceinline__ KeyT key_of(const Entry<1>& e) { return e.k[0]; }
    static __device__ __forceinline__ void set_key(Entry<1>& e, KeyT k) { e.k[0] = k; }

    static __device__ void load(Ctx& c, const InstDesc& d) {
        if (threadIdx.x == 0) {
            c.w = d.weights;
            c.W = d.W;
            c.H = d.H;
            c.goal = (uint32_t)d.goal0;
            c.start = (uint32_t)d.start0;
            c.gx = c.goal % d.W;
            c.gy = c.goal / d.W;
            c.minw = d.minw;
            c.href = d.heuristic;
        }
        __syncthreads();
    }
    static __device__ __forceinline__ Tab make_tab(const InstDesc& d) { return Tab{d.table}; }
    static __device__ __forceinline__ uint64_t get(const Tab& t, KeyT k) { return __ldcg(t.v + k); }
    static __device__ __forceinline__ uint32_t start_f(const Ctx&, const InstDesc& d) { return d.f0; }
    static constexpr uint32_t kRootCode = kRootMove;
    static constexpr bool kParentBySlot = false;
    struct Look {
        uint64_t v;
    };
    static __device__ __forceinline__ Look look_begin(const Tab& t, KeyT k) { return Look{__ldcg(t.v + k)}; }
    static __device__ __forceinline__ uint64_t look_end(const Tab&, KeyT, const Look& l) { return l.v; }
    static __device__ __forceinline__ uint64_t get_self(const Tab& t, KeyT k, uint32_t&) { return get(t, k); }
    static __device__ __forceinline__ uint32_t code(int m, uint32_t) { return (uint32_t)m; }
    static __device__ __forceinline__ int insert(const Tab& t, KeyT k, uint64_t v, uint64_t& old,
                                                 uint64_t& slot) {
        old = atomicMin(t.v + k, v);
        slot = k;
        return old == kEmpty ? 1 : 0;
    }
    static constexpr bool kDense = true;
    // The cell is the slot: one atomicMin claims and lowers it.
    static __device__ __forceinline__ int claim_first(const Tab& t, KeyT k, uint64_t v, uint64_t& slot,
                                                      uint64_t& old) {
        slot = k;
        old = atomicMin(t.v + k, v);
        return old == kEmpty ? 1 : 0;
    }
    static __device__ __forceinline__ int claim_probe(const Tab&, KeyT, uint64_t, uint64_t&, uint64_t&) {
        return -1;
    }
    static __device__ __forceinline__ uint64_t min_at(const Tab& t, uint64_t slot, KeyT, uint64_t v, uint64_t) {
        return atomicMin(t.v + slot, v);
    }
    static __device__ __forceinline__ bool is_goal(const Ctx& c, KeyT k) { return k == c.goal; }
    static __device__ __forceinline__ bool is_start(const Ctx& c, KeyT k) { return k == c.start; }
    // The eight neighbours' weights load together, before any successor
    // needs one (every load is inside the board, whatever k holds).
    static __device__ __forceinline__ Pre prepare(const Ctx& c, KeyT k) {
        const uint32_t cell = (uint32_t)k;
        Pre p{(int)(cell % c.W), (int)(cell / c.W), 0};
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const int nx = p.x + dx(m), ny = p.y + dy(m);
            if (nx >= 0 && ny >= 0 && nx < (int)c.W && ny < (int)c.H)
                p.wts |= (uint64_t)__ldg(c.w + (uint32_t)ny * c.W + (uint32_t)nx) << (8 * m);
        }
        return p;
    }
    static __device__ __forceinline__ uint32_t heur(const Ctx& c, int x, int y) {
        // 0: Chebyshev x min weight (admissible); 1: Manhattan (the reference's,
        // a_star_pathfinding.h:219-221); 2: zero.
        const uint32_t ax = (uint32_t)abs(x - (int)c.gx), ay = (uint32_t)abs(y - (int)c.gy);
        if (c.href == 1) return ax + ay;
        if (c.href == 2) return 0;
        return (ax > ay ? ax : ay) * c.minw;
    }
    static __device__ __forceinline__ bool succ(const Ctx& c, KeyT, Pre p, int m, uint32_t pm,
                                                uint32_t g, uint32_t, KeyT& nk, uint32_t& ng,
                                                uint32_t& nh) {
        if (pm != kRootMove && (uint32_t)m == inv(pm)) return false;
        const uint32_t wt = (uint32_t)(p.wts >> (8 * m)) & 0xffu;
        if (!wt) return false;  // obstacle or off the board
        const int nx = p.x + dx(m), ny = p.y + dy(m);
        const uint32_t cell = (uint32_t)ny * c.W + (uint32_t)nx;
        nk = cell;
        ng = g + wt;
        nh = heur(c, nx, ny);
        return true;
    }
    static __device__ __forceinline__ KeyT parent(const Ctx& c, const Tab&, KeyT k, uint32_t m) {
        return (KeyT)((int64_t)k - dx((int)m) - (int64_t)dy((int)m) * (int64_t)c.W);
    }
};

// ---------------------------------------------------------------------------
// Block-shared state.
// ---------------------------------------------------------------------------
struct CtaShared {
    TeamSlot slot[kSlots];  // team slots of a one-block team
    TeamSlot agg;           // this block's share of the current iteration (multi-block teams)
    unsigned long long agg_minprio;  // this block's heaps' min after the previous push
    unsigned long long cnt[5];       // expansions, stale, generated, pushes, claims of this block
                                     // in this launch (added to the control block at exit)
    unsigned long long pub[2];       // claims, expansions as of the last published cut
    unsigned long long run[2];       // claims, expansions of the cuts tested so far
    unsigned long long base[2];      // claims, expansions before this launch
    unsigned long long t_start;      // search start on the device clock
    uint32_t agg_err_prev;           // heap full in the previous push
    uint32_t dec_status, dec_best, dec_fmin, push_count;  // thread 0 -> block
    InstDesc desc;
    uint32_t inst, ok, slice, pad1;  // slice: iterations before suspending (0 = to the end)
    union {
        SlidingDom<3>::Ctx s3;
        SlidingDom<4>::Ctx s4;
        SlidingDom<5>::Ctx s5;
        GridDom::Ctx g;
    } ctx;
};

extern __shared__ uint4 g_dyn_smem[];

// Barrier over the blocks of a multi-block team: one atomic arrival on a
// counter that only grows, a poll until it reaches the end of this barrier's
// range, a bounded wait (deadline on the device clock), and an abort flag so
// that one block giving up releases the others.
__device__ __forceinline__ bool team_sync_grid(TeamCtl* tc, uint32_t nctas, uint64_t timeout_ns,
                                               CtaShared& sm) {
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t ok = 1;
        // Release: the block's writes (ordered before thread 0 by the block
        // barrier) become visible before the arrival does.
        asm volatile("fence.acq_rel.gpu;" ::: "memory");
        const unsigned long long old = atomicAdd(&tc->arrive, 1ull);
        const unsigned long long target = (old / nctas + 1) * nctas;
        const volatile unsigned long long* va = &tc->arrive;
        const volatile uint32_t* vab = &tc->abort;
        if (*va < target) {
            const uint64_t t0 = globaltimer_ns();
            for (uint32_t spin = 1;; ++spin) {
                if (*va >= target) break;
                if (*vab) {
                    ok = 0;
                    break;
                }
                if ((spin & 255u) == 0 && globaltimer_ns() - t0 > timeout_ns) {
                    atomicExch(&tc->abort, 1u);
                    ok = 0;
                    break;
                }
                if (spin > 64) __nanosleep(32);
            }
        }
        // Acquire: the other blocks' writes before their arrivals are visible.
        asm volatile("fence.acq_rel.gpu;" ::: "memory");
        if (*vab) ok = 0;
        sm.ok = ok;
    }
    __syncthreads();
    return sm.ok != 0;
}

__device__ __forceinline__ uint32_t ld_vol(const uint32_t* p) { return *(const volatile uint32_t*)p; }
__device__ __forceinline__ uint64_t ld_vol64(const unsigned long long* p) {
    return *(const volatile unsigned long long*)p;
}

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
// Strong relaxed reads: followed by fence_acq_rel_gpu they form acquire
// patterns.  Strong relaxed writes: after fence_acq_rel_gpu they form release
// patterns.
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void red_relaxed_add_u32(uint32_t* p, uint32_t v) {
    asm volatile("red.relaxed.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Waits (one thread) until the ready word *p carries iteration `target`
// (high half >= target), given `w`, a value of *p read before and ordered by
// an acquire fence since; returns the word in `w`.  Bounded like
// team_wait_u32 below; returns with acquire ordering.
__device__ __forceinline__ bool team_wait_ready(const unsigned long long* p, uint32_t target,
                                                unsigned long long& w, TeamCtl* tc, uint64_t timeout_ns) {
    if ((uint32_t)(w >> 32) >= target) return true;
    const volatile uint32_t* vab = &tc->abort;
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t spin = 1;; ++spin) {
        w = ld_acquire_u64(p);
        if ((uint32_t)(w >> 32) >= target) return true;
        if (*vab) return false;
        if ((spin & 255u) == 0 && globaltimer_ns() - t0 > timeout_ns) {
            atomicExch(&tc->abort, 1u);
            return false;
        }
        if (spin > 64) __nanosleep(32);
    }
}

// Waits (one thread) until *p >= target, given `seen`, a value of *p read
// before and ordered by an acquire fence since: bounded by the deadline,
// released by the team's abort flag; a timeout raises the flag.  Returns with
// acquire ordering: the writes the waited-for block made before raising *p
// are visible.
__device__ __forceinline__ bool team_wait_u32(const uint32_t* p, uint32_t target, uint32_t seen, TeamCtl* tc,
                                              uint64_t timeout_ns) {
    if (seen >= target) return true;
    const volatile uint32_t* vab = &tc->abort;
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t spin = 1;; ++spin) {
        if (ld_acquire_u32(p) >= target) return true;
        if (*vab) return false;
        if ((spin & 255u) == 0 && globaltimer_ns() - t0 > timeout_ns) {
            atomicExch(&tc->abort, 1u);
            return false;
        }
        if (spin > 64) __nanosleep(32);
    }
}

// The blocks working on one instance.
struct TeamRef {
    uint32_t ctas;  // blocks in the team (1 = one block, barriers are __syncthreads)
    uint32_t rank;  // this block's rank in the team
    TeamCtl* ctl;   // control block of a multi-block team (device)
    void* stage;    // stage buffers of a multi-block team (device)
};

// Inclusive warp prefix sum.
__device__ __forceinline__ uint32_t warp_incl_sum(uint32_t v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, v, o);
        if (lane >= o) v += t;
    }
    return v;
}
__device__ __forceinline__ uint64_t warp_min64(uint64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t t = __shfl_xor_sync(kFull, v, o);
        v = t < v ? t : v;
    }
    return v;
}


template <class D>
__device__ __noinline__ void run_instance(const LaunchParams& P, const InstDesc& d, CtaShared& sm,
                                          typename D::Ctx& ctx, const TeamRef tm) {
    constexpr int KW = D::KW;
    constexpr int MAXN = D::MAXN;
    using E = Entry<KW>;
    using KeyT = typename D::KeyT;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, W = blockDim.x >> 5;
    const bool multi = tm.ctas > 1;
    const uint32_t rank = tm.rank;
    const uint32_t H = d.heaps;
    TeamSlot* slots = sm.slot;  // one-block teams
    const uint32_t ew_cap = d.ew_wide > d.ew ? d.ew_wide : d.ew;  // widest pop of the search
    const size_t stage_cap = stage_entries_per_buffer(H, ew_cap, MAXN);
    char* dyn = reinterpret_cast<char*>(g_dyn_smem);
    E* const stage0 = multi ? reinterpret_cast<E*>(tm.stage) : reinterpret_cast<E*>(dyn);  // ring (multi)
    E* const snodes_all = reinterpret_cast<E*>(dyn + (multi ? 0 : 2 * stage_cap * sizeof(E)));
    InstCtl* ctl = d.ctl;
    const bool leader = rank == 0 && threadIdx.x == 0;

    auto tsync = [&]() -> bool {
        if (!multi) {
            __syncthreads();
            return true;
        }
        return team_sync_grid(tm.ctl, tm.ctas, P.barrier_timeout_ns, sm);
    };

    D::load(ctx, d);
    const typename D::Tab tab = D::make_tab(d);

    WarpHeap<KW> hp;
    const uint32_t hid = rank * W + warp;
    hp.nodes = reinterpret_cast<E*>(d.heap_nodes) + (size_t)hid * (d.heap_cap + 1) * 32;
    hp.sn = P.heap_snodes ? P.heap_snodes : kHeapSmemNodes;
    hp.snodes = snodes_all + (size_t)warp * (hp.sn - 1) * 32;
    hp.hdr = d.heap_hdr + 2 * hid;
    hp.cap = d.heap_cap;
    // Bucket front: pages, links and free stacks in the instance's bucket
    // area; the push scratch (64 words per warp) in shared memory after the
    // heap nodes.
    Buckets<KW> bq;
    {
        const uint32_t BP = P.buckets ? d.bq_pages : 0u;
        E* const pages_all = reinterpret_cast<E*>(d.bq_base);
        uint32_t* const link_all = reinterpret_cast<uint32_t*>(pages_all + (size_t)H * BP * 32);
        bq.P = BP;
        bq.pages = pages_all + (size_t)hid * BP * 32;
        bq.link = link_all + (size_t)hid * BP;
        bq.fstack = link_all + (size_t)H * BP + (size_t)hid * BP;
        bq.state = link_all + 2 * (size_t)H * BP + (size_t)hid * kBucketStateWords;
        bq.upd = reinterpret_cast<uint32_t*>(snodes_all + (size_t)W * (hp.sn - 1) * 32) + (size_t)warp * 64;
        bq_init(bq, lane);
    }

    const uint32_t life = ld_vol(&ctl->life);
    if (!multi && threadIdx.x < kSlots) {
        TeamSlot& t = sm.slot[threadIdx.x];
        t.minprio = kInfPrio;
        t.minstage = kInfPrio;
        t.count = 0;
        t.best = kInf;
        t.err = 0;
    }
    uint32_t status = kInf;  // kInf while running / suspended
    uint32_t best_r;         // best goal cost seen (identical in every thread)
    bool have_prev;          // the previous iteration's slot holds the heaps' min
    if (life == LIFE_FRESH) {
        // Clear the table (0xff = empty key and value) across the whole team:
        // only the slots the previous solve claimed when they were recorded
        // (a length above the list's capacity means they were not) and few,
        // otherwise the whole table.  Listed offsets are the previous solve's, in the
        // same buffer; its table may have been larger than this solve's.
        const uint64_t stride = (uint64_t)tm.ctas * blockDim.x;
        const uint64_t tid = (uint64_t)rank * blockDim.x + threadIdx.x;
        // Where either clear will do, scattered stores costing about a
        // 32-byte sector each against streaming ones, the list is used while
        // it covers under a quarter of the table's words.
        const uint64_t cnt = d.touched ? ld_vol64(d.touched_count) : 0;
        if (d.touched && cnt <= d.touched_cap &&
            (!d.clear_either || cnt * d.prev_slot_words * 4 < d.table_words)) {
            for (uint64_t i = tid; i < cnt; i += stride) {
                const uint32_t w = __ldcg(d.touched + i);
                if (w == kTouchedHole) continue;
                for (uint32_t j = 0; j < d.prev_slot_words; ++j) __stcg(d.table + w + j, kEmpty);
            }
        } else {
            uint4* tp = reinterpret_cast<uint4*>(d.table);
            const uint64_t n16 = d.table_words / 2;
            for (uint64_t i = tid; i < n16; i += stride) __stcg(tp + i, make_uint4(~0u, ~0u, ~0u, ~0u));
            if ((d.table_words & 1) && tid == 0)  // odd cell count: last word
                __stcg(d.table + d.table_words - 1, kEmpty);
        }
        heap_init(hp);
        if (!tsync()) status = ST_BARRIER;
        if (hid == 0) {
            E s = inf_entry<KW>();
            s.prio = make_prio(D::start_f(ctx, d), 0, kRootMove);
            D::set_key(s, ctx.start);
            if (lane == 0) hp.part = s;
            hp.pc = 1;
        }
        if (leader) {
            uint64_t old, slot = 0;
            D::insert(tab, ctx.start, make_val(0, D::kRootCode), old, slot);
            if (d.touched) {
                *d.touched_count = 1;
                d.touched[0] = (uint32_t)slot;
            }
            atomicAdd(&ctl->table_used, 1ull);
            ctl->t_start = globaltimer_ns();
        }
        best_r = D::is_goal(ctx, ctx.start) ? 0u : kInf;
        have_prev = true;  // the start is the only open entry; every slot starts empty
    } else {
        heap_restore(hp, lane);
        bq_restore(bq, lane);
        best_r = ld_vol(&ctl->best);
        have_prev = false;
    }
    // Multi-block teams: each block stages into its own region of the ring
    // buffers and aggregates its counters and minima in shared memory; thread
    // 0 publishes them (ready word, cut slot).
    const size_t region_cap = stage_entries_per_buffer(W, ew_cap, MAXN);
    unsigned long long* const ready =
        multi ? reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(tm.stage) +
                                                      (size_t)kStageRing * stage_cap * sizeof(E))
              : nullptr;
    if (multi && threadIdx.x == 0) {
        for (uint32_t r = 0; r < kStageRing; ++r) ready[(size_t)r * tm.ctas + rank] = 0;
        if (rank == 0)
            for (uint32_t k = 0; k < kCuts; ++k) {
                CutSlot& c = tm.ctl->cut[k];
                c.minprio = kInfPrio;
                c.claims = c.exps = 0;
                c.best = kInf;
                c.lossy = c.err = c.count = 0;
            }
    }
    if (status == kInf && !tsync()) status = ST_BARRIER;

    const uint32_t ew = d.ew;
    // This warp's current claim-list chunk (none reserved yet).
    unsigned long long t_base = 0;
    uint32_t t_used = kTouchedChunk;
    uint32_t fmin = D::start_f(ctx, d);  // min f over the open list at the last check
    uint32_t it = 0;
    const uint32_t it0 = ld_vol(&ctl->iterations);
    if (threadIdx.x == 0) {
        sm.agg.minstage = kInfPrio;
        sm.agg.best = kInf;
        sm.agg.err = 0;
        sm.agg.count = 0;
        sm.agg_minprio = kInfPrio;
        sm.agg_err_prev = 0;
        for (int i = 0; i < 5; ++i) sm.cnt[i] = 0;
        // Budgets are tested against these (no global reads per iteration).
        sm.base[0] = ld_vol64(&ctl->table_used);
        sm.base[1] = ld_vol64(&ctl->expansions);
        sm.t_start = *(const volatile uint64_t*)&ctl->t_start;
        sm.pub[0] = sm.pub[1] = sm.run[0] = sm.run[1] = 0;
    }
    __syncthreads();
    // The first cut of a multi-block team holds the heaps as they are now.
    if (multi) {
        const uint64_t mp = open_min(hp, bq);
        if (lane == 0 && mp != kInfPrio) atomicMin(&sm.agg_minprio, (unsigned long long)mp);
    }
    while (status == kInf) {
        const uint32_t s = it % kSlots;
        TeamSlot* S = slots + s;
        // Where this block's warps record the iteration: the team slot itself
        // for one-block teams (shared memory), the block aggregate otherwise.
        TeamSlot* Sw = multi ? &sm.agg : S;
        E* const stage = multi ? stage0 + ((size_t)(it % kStageRing) * tm.ctas + rank) * region_cap
                               : stage0 + (size_t)(it & 1) * stage_cap;
        if (!multi && leader) {
            // One-block team: slot it+1 was last read right after the block
            // barrier of iteration it-2; every warp is past that point, and
            // none writes it before the barrier of this iteration.
            TeamSlot* nx = slots + (it + 1) % kSlots;
            nx->minprio = kInfPrio;
            nx->minstage = kInfPrio;
            nx->count = 0;
            nx->best = kInf;
            nx->err = 0;
            if (sm.base[0] + sm.cnt[4] > d.table_limit) atomicCAS(&S->err, 0u, (uint32_t)ST_TABLE_FULL);
            if (d.max_exp && sm.base[1] + sm.cnt[0] >= d.max_exp) atomicCAS(&S->err, 0u, (uint32_t)ST_BUDGET);
            if (d.max_iter && it0 + it + 1 >= d.max_iter) atomicCAS(&S->err, 0u, (uint32_t)ST_BUDGET);
            if (d.timeout_ns && globaltimer_ns() - sm.t_start > d.timeout_ns)
                atomicCAS(&S->err, 0u, (uint32_t)ST_TIMEOUT);
        }

        // ---- pop: up to ew entries per warp-heap, inside the window ----
        // With delta set, only entries with f <= fmin + delta are expanded
        // (delta-stepping); the rest wait for later iterations.
        const uint64_t lim = (d.delta && (uint64_t)fmin + d.delta < 0xffffffffull)
                                 ? ((uint64_t)(fmin + d.delta + 1) << 32)
                                 : kInfPrio;
        E e;
        const uint32_t cnt =
            open_pop(hp, bq, d.wide_after && it0 + it >= d.wide_after ? d.ew_wide : ew, lim, e, lane);
        bool act = (uint32_t)lane < cnt;
        const KeyT k = D::key_of(e);
        const uint32_t g = prio_g(e.prio), h = prio_f(e.prio) - g;
        uint32_t pm = prio_pm(e.prio), self = 0;
        bool stale = false;
        uint32_t goal_g = kInf;
        if (act && D::is_goal(ctx, k)) {
            // The goal is never expanded (a_star.h:80-83); its cost counts
            // unless a lower g for it is already known.
            if ((uint32_t)(D::get(tab, k) >> 32) >= g) goal_g = g;
            act = false;
        }
        typename D::Look look{};
        if constexpr (D::kParentBySlot) {
            // Plugins record parents by slot: the entry's own slot is needed
            // before its successors are inserted.
            if (act) {
                const uint64_t v = D::get_self(tab, k, self);
                pm = (uint32_t)v;
                if ((uint32_t)(v >> 32) < g) {
                    stale = true;
                    act = false;
                }
            }
        } else {
            if (act) look = D::look_begin(tab, k);  // resolved after the probes are in flight
        }

        // ---- expand: per group of moves, all successors, then all probes,
        // then all atomicMins, so each group costs ~2 memory round trips ----
        const typename D::Pre pre = D::prepare(ctx, k);
        constexpr int GS = MAXN < 4 ? MAXN : 4;
        uint32_t n_gen = 0, n_claim = 0, pushed = 0;
        uint64_t smin = kInfPrio;
        bool tfull = false, range = false;
#pragma unroll
        for (int g0 = 0; g0 < MAXN; g0 += GS) {
            KeyT nk[GS];
            uint32_t ng[GS], nh[GS];
            bool ok[GS];
#pragma unroll
            for (int j = 0; j < GS; ++j) {
                ok[j] = act && D::succ(ctx, k, pre, g0 + j, pm, g, h, nk[j], ng[j], nh[j]);
                n_gen += ok[j];
                if (ok[j] && ng[j] > kMaxG) {
                    range = true;
                    ok[j] = false;
                }
                ok[j] = ok[j] && ng[j] + nh[j] < best_r;  // cannot beat the best goal found
            }
            uint64_t slot[GS], old[GS], val[GS];
            int cl[GS];
#pragma unroll
            for (int j = 0; j < GS; ++j) {
                val[j] = make_val(ng[j], D::code(g0 + j, self));
                old[j] = 0;
                cl[j] = ok[j] ? D::claim_first(tab, nk[j], val[j], slot[j], old[j]) : -1;
            }
#pragma unroll
            for (int j = 0; j < GS; ++j) {
                if (cl[j] == 2) cl[j] = D::claim_probe(tab, nk[j], val[j], slot[j], old[j]);
                if (ok[j] && cl[j] < 0) tfull = true;
            }
#pragma unroll
            for (int j = 0; j < GS; ++j) {
                if (cl[j] >= kClNeedMin) {
                    old[j] = D::min_at(tab, slot[j], nk[j], val[j], old[j]);
                    cl[j] -= kClNeedMin;
                }
            }
            if constexpr (!D::kParentBySlot) {
                if (g0 == 0 && act && (uint32_t)(D::look_end(tab, k, look) >> 32) < g) {
                    // Stale: the table g went below the entry's own.  The
                    // successors just inserted are real paths and stay in the
                    // table but are not queued; the entry with the lower g
                    // covers them.
                    stale = true;
                    act = false;
                }
            }
            uint32_t nacc = 0, ncl = 0;
            bool acc[GS], clm[GS];
#pragma unroll
            for (int j = 0; j < GS; ++j) {
                const bool in = ok[j] && cl[j] >= 0;
                acc[j] = in && act && (uint32_t)(old[j] >> 32) > ng[j];
                clm[j] = in && cl[j] == 1;
                nacc += acc[j];
                ncl += clm[j];
                if (acc[j]) {
                    const uint64_t pr = make_prio(ng[j] + nh[j], ng[j], (uint32_t)(g0 + j));
                    smin = pr < smin ? pr : smin;
                    if (D::is_goal(ctx, nk[j]) && ng[j] < goal_g) goal_g = ng[j];
                }
            }
            n_claim += ncl;
            // Stage the improved successors: one atomic per warp reserves the range.
            const uint32_t incl = warp_incl_sum(nacc, lane);
            const uint32_t total = __shfl_sync(kFull, incl, 31);
            if (total) {
                uint32_t base = 0;
                if (lane == 31) base = atomicAdd(&Sw->count, total);
                base = __shfl_sync(kFull, base, 31) + incl - nacc;
#pragma unroll
                for (int j = 0; j < GS; ++j) {
                    if (acc[j]) {
                        E out = inf_entry<KW>();
                        out.prio = make_prio(ng[j] + nh[j], ng[j], (uint32_t)(g0 + j));
                        D::set_key(out, nk[j]);
                        st_stage(stage + base++, out, multi);
                    }
                }
                pushed += total;
            }
            if (d.touched) {  // record claimed slots for the next solve's clear
                const uint32_t ci = warp_incl_sum(ncl, lane);
                const uint32_t ct = __shfl_sync(kFull, ci, 31);
                if (ct) {
                    // Fill the warp's chunk; a group that overruns it
                    // continues in a newly reserved one.
                    const uint32_t room = kTouchedChunk - t_used;
                    unsigned long long nb = 0;
                    if (ct > room) {
                        if (lane == 0) nb = atomicAdd(d.touched_count, (unsigned long long)kTouchedChunk);
                        nb = __shfl_sync(kFull, nb, 0);
                    }
                    uint32_t pos = ci - ncl;
#pragma unroll
                    for (int j = 0; j < GS; ++j) {
                        if (clm[j]) {
                            const unsigned long long at = pos < room ? t_base + t_used + pos : nb + (pos - room);
                            if (at < d.touched_cap) d.touched[at] = (uint32_t)slot[j];
                            ++pos;
                        }
                    }
                    if (ct > room) {
                        t_base = nb;
                        t_used = ct - room;
                    } else {
                        t_used += ct;
                    }
                }
            }
        }
        const unsigned bexp = __ballot_sync(kFull, act), bstale = __ballot_sync(kFull, stale);
        {
            uint32_t gsum = n_gen, csum = n_claim;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                gsum += __shfl_xor_sync(kFull, gsum, o);
                csum += __shfl_xor_sync(kFull, csum, o);
                const uint32_t gg = __shfl_xor_sync(kFull, goal_g, o);
                goal_g = gg < goal_g ? gg : goal_g;
            }
            smin = warp_min64(smin);
            const bool any_full = __any_sync(kFull, tfull), any_range = __any_sync(kFull, range);
            if (lane == 0) {
                if (bexp) atomicAdd(&sm.cnt[0], (unsigned long long)__popc(bexp));
                if (bstale) atomicAdd(&sm.cnt[1], (unsigned long long)__popc(bstale));
                if (gsum) atomicAdd(&sm.cnt[2], (unsigned long long)gsum);
                if (pushed) atomicAdd(&sm.cnt[3], (unsigned long long)pushed);
                if (csum) atomicAdd(&sm.cnt[4], (unsigned long long)csum);
                if (smin != kInfPrio) atomicMin(&Sw->minstage, (unsigned long long)smin);
                if (goal_g != kInf) atomicMin(&Sw->best, goal_g);
                if (any_full) atomicCAS(&Sw->err, 0u, (uint32_t)ST_TABLE_FULL);
                if (any_range) atomicCAS(&Sw->err, 0u, (uint32_t)ST_COST_RANGE);
            }
        }
        if (multi) {
            // ---- one hand-off per iteration: publish cut `it` and this
            // block's stage region, then wait for the region this block
            // pushes and test cut it - kCutLag (a_star.h:260-262) ----
            __syncthreads();  // every warp's stage writes and counters are done
            if (threadIdx.x == 0) {
                CutSlot* cuts = tm.ctl->cut;
                unsigned long long* const rw = ready + (size_t)(it % kStageRing) * tm.ctas;
                const uint32_t from = (rank + it) % tm.ctas;
                // Both awaited words are read first, relaxed (the fence below
                // orders them before what follows): their round trips overlap
                // this block's publication.
                unsigned long long wfrom = from == rank ? 0ull : ld_relaxed_u64(rw + from);
                const CutSlot* t = cuts + (it + kCuts - kCutLag) % kCuts;
                const uint32_t tseen = it >= kCutLag ? ld_relaxed_u32(&t->count) : 0u;
                const uint32_t lossy = sm.agg.err ? sm.agg.err : sm.agg_err_prev;
                uint32_t err = 0;
                if (leader) {
                    if (it >= 2 * kCutLag + 2) {  // every block has read it; none writes it yet
                        CutSlot* r = cuts + (it - 2 * kCutLag - 2) % kCuts;
                        r->minprio = kInfPrio;
                        r->claims = r->exps = 0;
                        r->best = kInf;
                        r->lossy = r->err = r->count = 0;
                    }
                    if (d.max_iter && it0 + it + 1 >= d.max_iter) err = ST_BUDGET;
                    if (d.timeout_ns && globaltimer_ns() - sm.t_start > d.timeout_ns) err = ST_TIMEOUT;
                }
                // Cut `it` covers this block's heaps after the previous push
                // (a superset of what is left after this iteration's pops) and
                // what this iteration staged.
                CutSlot* c = cuts + it % kCuts;
                const unsigned long long cm =
                    sm.agg_minprio < sm.agg.minstage ? sm.agg_minprio : sm.agg.minstage;
                if (cm != kInfPrio) atomicMin(&c->minprio, cm);
                if (sm.cnt[4] != sm.pub[0]) atomicAdd(&c->claims, sm.cnt[4] - sm.pub[0]);
                if (sm.cnt[0] != sm.pub[1]) atomicAdd(&c->exps, sm.cnt[0] - sm.pub[1]);
                sm.pub[0] = sm.cnt[4];
                sm.pub[1] = sm.cnt[0];
                if (sm.agg.best != kInf) atomicMin(&c->best, sm.agg.best);
                if (lossy) atomicCAS(&c->lossy, 0u, lossy);
                if (err) atomicCAS(&c->err, 0u, err);
                const uint32_t mine = sm.agg.count;
                // One fence for both arrivals and both early reads: every
                // warp's stage writes (ordered before thread 0 by the block
                // barrier) and the cut's updates precede the ready word and
                // the cut arrival (release); the words read above precede
                // everything after (acquire).
                fence_acq_rel_gpu();
                st_relaxed_u64(rw + rank, ((unsigned long long)(it + 1) << 32) | mine);
                red_relaxed_add_u32(&c->count, 1u);
                sm.agg.best = kInf;
                sm.agg.err = 0;
                sm.agg.count = 0;
                sm.agg.minstage = kInfPrio;
                sm.agg_minprio = kInfPrio;
                sm.agg_err_prev = 0;
                uint32_t dec = kInf, n = 0, dbest = kInf, dfmin = kInf;
                if (from == rank)
                    n = mine;
                else if (!team_wait_ready(rw + from, it + 1, wfrom, tm.ctl, P.barrier_timeout_ns))
                    dec = ST_BARRIER;
                else
                    n = (uint32_t)wfrom;
                if (dec == kInf && it >= kCutLag) {
                    // Waits only while a block is more than kCutLag iterations behind.
                    if (!team_wait_u32(&t->count, tm.ctas, tseen, tm.ctl, P.barrier_timeout_ns)) {
                        dec = ST_BARRIER;
                    } else {
                        const uint64_t open_min = ld_vol64(&t->minprio);
                        dbest = ld_vol(&t->best);
                        uint32_t tl = ld_vol(&t->lossy), te = ld_vol(&t->err);
                        // Budgets from the team's totals, the same in every block.
                        sm.run[0] += ld_vol64(&t->claims);
                        sm.run[1] += ld_vol64(&t->exps);
                        if (!tl && sm.base[0] + sm.run[0] > d.table_limit) tl = ST_TABLE_FULL;
                        if (!te && d.max_exp && sm.base[1] + sm.run[1] >= d.max_exp) te = ST_BUDGET;
                        const uint32_t bb = dbest < best_r ? dbest : best_r;
                        if (tl) dec = tl;  // an iteration that lost entries proves nothing
                        else if (bb != kInf && bb <= prio_f(open_min)) dec = ST_OK;
                        else if (te) dec = te;
                        else if (open_min == kInfPrio) dec = ST_NO_PATH;
                        if (open_min != kInfPrio) dfmin = prio_f(open_min);
                    }
                }
                sm.dec_status = dec;
                sm.dec_best = dbest;
                sm.dec_fmin = dfmin;
                sm.push_count = n;
            }
            __syncthreads();
            {
                const uint32_t db = sm.dec_best;
                best_r = db < best_r ? db : best_r;
                if (sm.dec_fmin != kInf) fmin = sm.dec_fmin;
                status = sm.dec_status;
            }
            if (status != kInf) break;
        } else {
            if (!tsync()) {
                status = ST_BARRIER;
                break;
            }
            // ---- termination test (a_star.h:260-262), one iteration behind ----
            // Open entries now: heaps after the previous push (>= that slot's
            // min) minus this iteration's pops, plus this iteration's stage.
            const uint32_t sb = ld_vol(&S->best);
            best_r = sb < best_r ? sb : best_r;
            uint32_t err = ld_vol(&S->err);
            uint64_t open_min = ld_vol64(&S->minstage);
            if (have_prev) {
                const TeamSlot* pv = slots + (it + kSlots - 1) % kSlots;
                if (!err) err = ld_vol(&pv->err);
                const uint64_t mp = ld_vol64(&pv->minprio);
                open_min = mp < open_min ? mp : open_min;
            }
            // An iteration that lost entries (full table or heap) proves nothing.
            if (err == ST_TABLE_FULL || err == ST_HEAP_FULL || err == ST_COST_RANGE) status = err;
            else if (have_prev && best_r != kInf && best_r <= prio_f(open_min)) status = ST_OK;
            else if (err) status = err;
            else if (have_prev && open_min == kInfPrio) status = ST_NO_PATH;
            if (status != kInf) break;
            if (open_min != kInfPrio) fmin = prio_f(open_min);
        }

        // ---- push ----
        // One-block teams deal the block's stage chunks round-robin with a
        // rotating offset; in a multi-block team block r takes the region of
        // block (r + it) mod blocks, so work moves between blocks every
        // iteration, and its warps deal that region's chunks.
        {
            uint32_t total;
            const E* src;
            uint32_t first, step;
            if (multi) {
                const uint32_t from = (rank + it) % tm.ctas;
                total = sm.push_count;
                src = stage0 + ((size_t)(it % kStageRing) * tm.ctas + from) * region_cap;
                first = ((uint32_t)warp + it) % (uint32_t)W;
                step = (uint32_t)W;
            } else {
                total = ld_vol(&S->count);
                src = stage;
                first = (hid + H - it % H) % H;
                step = H;
            }
            const uint32_t nch = (total + 31) / 32;
            bool hfull = false;
            for (uint32_t c = first; c < nch; c += step) {
                const uint32_t idx = c * 32 + (uint32_t)lane;
                E x = idx < total ? ld_stage(src + idx, multi) : inf_entry<KW>();
                const uint32_t m = total - c * 32 < 32 ? total - c * 32 : 32;
                if (!open_push(hp, bq, x, m, lane)) {
                    hfull = true;
                    break;
                }
            }
            const uint64_t mp = open_min(hp, bq);
            if (lane == 0) {
                if (multi) {
                    atomicMin(&sm.agg_minprio, (unsigned long long)mp);
                    if (hfull) atomicCAS(&sm.agg_err_prev, 0u, (uint32_t)ST_HEAP_FULL);
                } else {
                    atomicMin(&S->minprio, (unsigned long long)mp);
                    if (hfull) atomicCAS(&S->err, 0u, (uint32_t)ST_HEAP_FULL);
                }
            }
        }
        ++it;
        have_prev = true;
        if (sm.slice && it >= sm.slice) break;  // suspend
    }

    if (lane == 0) atomicMax(&ctl->max_nodes, hp.max_n);
    if (d.touched)  // the unused rest of the warp's chunk
        for (uint32_t i = t_used + (uint32_t)lane; i < kTouchedChunk; i += 32)
            if (t_base + i < d.touched_cap) d.touched[t_base + i] = kTouchedHole;
    {  // this launch's counters
        __syncthreads();
        if (threadIdx.x == 0) {
            if (sm.cnt[0]) atomicAdd(&ctl->expansions, sm.cnt[0]);
            if (sm.cnt[1]) atomicAdd(&ctl->stale, sm.cnt[1]);
            if (sm.cnt[2]) atomicAdd(&ctl->generated, sm.cnt[2]);
            if (sm.cnt[3]) atomicAdd(&ctl->pushes, sm.cnt[3]);
            if (sm.cnt[4]) atomicAdd(&ctl->table_used, sm.cnt[4]);
            for (int i = 0; i < 5; ++i) sm.cnt[i] = 0;
        }
    }
    if (status == kInf) {
        // Suspending: fold in what the iterations not tested yet found -- a
        // goal popped there is in no heap any more -- and stop on entries
        // they lost.
        if (multi) {
            if (threadIdx.x == 0) {
                CutSlot* c = tm.ctl->cut + it % kCuts;
                if (sm.agg.best != kInf) atomicMin(&c->best, sm.agg.best);
                const uint32_t lossy = sm.agg.err ? sm.agg.err : sm.agg_err_prev;
                if (lossy) atomicCAS(&c->lossy, 0u, lossy);
            }
            if (!tsync()) {
                status = ST_BARRIER;
            } else {
                if (threadIdx.x == 0) {
                    uint32_t b = best_r, lossy = 0;
                    for (uint32_t x = it > kCutLag ? it - kCutLag : 0; x <= it; ++x) {
                        const CutSlot* c = tm.ctl->cut + x % kCuts;
                        const uint32_t cb = ld_vol(&c->best);
                        b = cb < b ? cb : b;
                        if (!lossy) lossy = ld_vol(&c->lossy);
                    }
                    sm.dec_best = b;
                    sm.dec_status = lossy ? lossy : kInf;
                }
                __syncthreads();
                best_r = sm.dec_best;
                status = sm.dec_status;
            }
        } else if (it > 0 && ld_vol(&slots[(it + kSlots - 1) % kSlots].err) == ST_HEAP_FULL) {
            status = ST_HEAP_FULL;  // raised by the last push
        }
    }
    if (status == kInf) {  // suspended: keep the search state resident
        heap_save(hp, lane);
        bq_save(bq, lane);
        if (leader) {
            ctl->best = best_r;
            ctl->iterations = it0 + it;
            __threadfence();
            ctl->life = LIFE_RUNNING;
        }
        return;
    }
    if (leader) {
        ctl->best = best_r;
        ctl->iterations = it0 + it;
        ctl->status = status;
        ctl->t_end = globaltimer_ns();
        __threadfence();
        ctl->life = LIFE_DONE;
    }
}

template <uint32_t KINDS>
__device__ __forceinline__ void dispatch(const LaunchParams& P, CtaShared& sm, const TeamRef tm) {
    switch (sm.desc.kind) {
        case KIND_SLIDING3:
            if constexpr ((KINDS & kind_bit(KIND_SLIDING3)) != 0) run_instance<SlidingDom<3>>(P, sm.desc, sm, sm.ctx.s3, tm);
            break;
        case KIND_SLIDING4:
            if constexpr ((KINDS & kind_bit(KIND_SLIDING4)) != 0) run_instance<SlidingDom<4>>(P, sm.desc, sm, sm.ctx.s4, tm);
            break;
        case KIND_SLIDING5:
            if constexpr ((KINDS & kind_bit(KIND_SLIDING5)) != 0) run_instance<SlidingDom<5>>(P, sm.desc, sm, sm.ctx.s5, tm);
            break;
        case KIND_GRID:
            if constexpr ((KINDS & kind_bit(KIND_GRID)) != 0) run_instance<GridDom>(P, sm.desc, sm, sm.ctx.g, tm);
            break;
        default:
            break;
    }
}

// Persistent search kernel.
//  * plain (team_ctas > 1): every block works on instance 0 (cooperative launch);
//  * batch/serve: blocks of the heavy teams first take heavy instances together,
//    then every block takes instances one block each from a work counter.
// MAXT bounds the block size: 256 threads (8 warps) leave the compiler up to
// 255 registers per thread, no spills; the all-kinds kernel has a second
// instantiation for 16-warp blocks (batch/serve), capped at 128 registers.
template <uint32_t KINDS, int MAXT = 256>
__global__ void __launch_bounds__(MAXT, 1) search_kernel(LaunchParams P) {
    __shared__ CtaShared sm;
    if (P.team_ctas > 1) {
        if (threadIdx.x == 0) {
            sm.desc = P.insts[0];
            sm.slice = P.slice_iters;
        }
        __syncthreads();
        dispatch<KINDS>(P, sm, TeamRef{P.team_ctas, blockIdx.x, P.team, P.stage});
        return;
    }
    if (P.n_heavy && blockIdx.x < P.heavy_teams * P.heavy_team) {
        const uint32_t t = blockIdx.x / P.heavy_team, rank = blockIdx.x % P.heavy_team;
        TeamCtl* tc = P.heavy_ctl + t;
        const TeamRef tm{P.heavy_team, rank, tc,
                         reinterpret_cast<char*>(P.heavy_stage) + (size_t)t * P.heavy_stage_bytes};
        for (;;) {
            // Every block of the team is done with the previous instance here.
            if (!team_sync_grid(tc, P.heavy_team, P.barrier_timeout_ns, sm)) break;
            if (rank == 0 && threadIdx.x == 0) {
                for (uint32_t k = 0; k < kCuts; ++k) {
                    tc->cut[k].minprio = kInfPrio;
                    tc->cut[k].claims = tc->cut[k].exps = 0;
                    tc->cut[k].best = kInf;
                    tc->cut[k].lossy = 0;
                    tc->cut[k].err = 0;
                    tc->cut[k].count = 0;
                }
                tc->inst = atomicAdd(P.heavy_next, 1u);
            }
            if (!team_sync_grid(tc, P.heavy_team, P.barrier_timeout_ns, sm)) break;
            const uint32_t i = ld_vol(&tc->inst);
            if (i >= P.n_heavy) break;
            if (threadIdx.x == 0) {
                const uint32_t slot = P.heavy_order[i];
                sm.desc = P.insts[slot];
                sm.slice = P.slices ? P.slices[slot] : P.slice_iters;
            }
            __syncthreads();
            dispatch<KINDS>(P, sm, tm);
        }
        __syncthreads();
    }
    for (;;) {
        if (threadIdx.x == 0) sm.inst = atomicAdd(P.next, 1u);
        __syncthreads();
        const uint32_t i = sm.inst;
        if (i >= P.n_insts) break;
        if (threadIdx.x == 0) {
            const uint32_t slot = P.order ? P.order[i] : i;
            sm.desc = P.insts[slot];
            sm.slice = P.slices ? P.slices[slot] : P.slice_iters;
        }
        __syncthreads();
        dispatch<KINDS>(P, sm, TeamRef{1, 0, nullptr, nullptr});
        __syncthreads();
    }
}

// Path rebuild (a_star.h:268-281 walked one <<<1,1>>> launch per step): for
// each finished puzzle one thread follows parent moves from the goal to the
// start and writes the states goal-first (grids: walk_grid_path, a warp per
// instance).  An instance that has the arena to itself (a launch of one)
// writes as it walks; otherwise it walks twice -- once to count, once to
// write into a slice of the shared arena reserved with one atomic.
template <class D>
__device__ void walk_path(const InstDesc& d, typename D::Ctx& ctx, unsigned long long* arena,
                          unsigned long long arena_words, unsigned long long* arena_used, bool own_arena,
                          unsigned long long base_off = 0) {
    InstCtl* ctl = d.ctl;
    const typename D::Tab tab = D::make_tab(d);
    // Every step lowers g by at least 1, so a walk longer than best + 1 states
    // means a damaged table.
    const uint64_t limit = (uint64_t)ctl->best + 2;
    if (own_arena) {
        const uint64_t cap = arena_words / D::KW;
        uint64_t len = 0;
        for (typename D::KeyT k = ctx.goal;;) {
            if (len >= cap || len > limit) {  // the host retries with room for best + 1 states
                ctl->status = ST_PATH_CAP;
                ctl->path_len = 0;
                return;
            }
            unsigned long long* o = arena + len * D::KW;
            o[0] = (uint64_t)k;
            if constexpr (D::KW == 2) o[1] = (uint64_t)(k >> 64);
            ++len;
            if (D::is_start(ctx, k)) break;
            const uint64_t v = D::get(tab, k);
            const uint32_t m = (uint32_t)v;
            if (v == kEmpty || m == D::kRootCode) {
                ctl->status = ST_PATH_CAP;
                ctl->path_len = 0;
                return;
            }
            k = D::parent(ctx, tab, k, m);
        }
        ctl->path_len = (uint32_t)len;
        ctl->path_off = base_off;
        atomicAdd(arena_used, (unsigned long long)(len * D::KW));
        return;
    }
    uint64_t len = 1;
    for (typename D::KeyT k = ctx.goal; !D::is_start(ctx, k); ++len) {
        const uint64_t v = D::get(tab, k);
        const uint32_t m = (uint32_t)v;
        if (v == kEmpty || m == D::kRootCode || len > limit) {
            ctl->status = ST_PATH_CAP;
            ctl->path_len = 0;
            return;
        }
        k = D::parent(ctx, tab, k, m);
    }
    const unsigned long long words = len * D::KW;
    const unsigned long long off = atomicAdd(arena_used, words);
    ctl->path_len = (uint32_t)len;
    if (off + words > arena_words) {
        ctl->status = ST_PATH_CAP;
        return;
    }
    ctl->path_off = off;
    typename D::KeyT k = ctx.goal;
    for (uint64_t i = 0; i < len; ++i) {
        unsigned long long* o = arena + off + i * D::KW;
        o[0] = (uint64_t)k;
        if constexpr (D::KW == 2) o[1] = (uint64_t)(k >> 64);
        if (i + 1 < len) k = D::parent(ctx, tab, k, (uint32_t)D::get(tab, k));
    }
}

// Builds the domain context without the block-wide table fill (one thread).
template <int N> __device__ void sliding_ctx_min(typename SlidingDom<N>::Ctx& c, const InstDesc& d) {
    c.goal = SlidingDom<N>::desc_key(d.goal0, d.goal1);
    c.start = SlidingDom<N>::desc_key(d.start0, d.start1);
}

// Grid path rebuild by one warp.  A dependent table load per step costs a
// DRAM round trip (~0.6 us; a 8192^2 grid's path has ~9k steps), so the warp
// loads the values of a kPathWin x kPathWin window of cells in one round
// trip (lane j reads column j of every row, 32 loads in flight) into shared
// memory, and lane 0 follows parent moves inside it.  Parents lead toward the
// start, so the window is placed with the current cell kPathMargin cells from
// its edge away from the start: up to ~28 steps per load.
constexpr int kPathWin = 32, kPathMargin = 3, kPathWarps = 4;
// GridDom::dx(m) + 1 and GridDom::dy(m) + 1 in bits 2m..2m+1.
constexpr uint32_t kGridDxPack = 2u | 0u << 2 | 1u << 4 | 1u << 6 | 2u << 8 | 2u << 10 | 0u << 12 | 0u << 14;
constexpr uint32_t kGridDyPack = 1u | 1u << 2 | 2u << 4 | 0u << 6 | 2u << 8 | 0u << 10 | 2u << 12 | 0u << 14;

static __device__ __forceinline__ int path_win_origin(int c, int s, int n) {
    int o = s < c ? c - (kPathWin - 1 - kPathMargin) : s > c ? c - kPathMargin : c - kPathWin / 2;
    if (o > n - kPathWin) o = n - kPathWin;
    return o < 0 ? 0 : o;
}

// Walks the grid path of `d` from the goal to the start (the whole warp
// calls it).  With `out`, lane 0 writes the cells goal-first, at most `cap`
// of them (`capped` is set when there were more).  Returns the number of
// states, or 0 for a damaged table: a cell without a move, a move leaving the
// grid, or more than `limit` states.
static __device__ uint64_t walk_grid_warp(const InstDesc& d, unsigned long long* win, unsigned long long* out,
                                   uint64_t cap, uint64_t limit, int lane, bool& capped) {
    const int W = (int)d.W, H = (int)d.H;
    const int sx = (int)(d.start0 % d.W), sy = (int)(d.start0 / d.W);
    int cx = (int)(d.goal0 % d.W), cy = (int)(d.goal0 / d.W);
    unsigned long long len = 0;
    int state = 0;  // 0: walking, 1: at the start, 2: damaged table
    bool cp = false;
    while (state == 0) {
        const int x0 = path_win_origin(cx, sx, W), y0 = path_win_origin(cy, sy, H);
        const int x = x0 + lane;
        unsigned long long v[kPathWin];
#pragma unroll
        for (int r = 0; r < kPathWin; ++r)
            v[r] = (x < W && y0 + r < H) ? __ldcg(d.table + (size_t)(y0 + r) * W + x) : kEmpty;
#pragma unroll
        for (int r = 0; r < kPathWin; ++r) win[r * kPathWin + lane] = v[r];
        __syncwarp();
        if (lane == 0) {
            // Window-local coordinates; a step is one shared-memory load and
            // a few integer operations (dx, dy from 2-bit fields).  Inside
            // the window a cell outside the grid holds kEmpty (loaded so), so
            // the grid bounds are checked only when the walk leaves it.
            int lx = cx - x0, ly = cy - y0;
            const int slx = sx - x0, sly = sy - y0;
            unsigned long long cell = (unsigned long long)cy * W + cx;
            for (;;) {
                if (out) {
                    if (len < cap) out[len] = cell;
                    else cp = true;
                }
                ++len;
                if (lx == slx && ly == sly) {
                    state = 1;
                    break;
                }
                const unsigned long long t = win[ly * kPathWin + lx];
                const uint32_t m = (uint32_t)t;
                if (len > limit || t == kEmpty || m >= 8) {
                    state = 2;
                    break;
                }
                const int dx = (int)((kGridDxPack >> (2 * m)) & 3u) - 1;
                const int dy = (int)((kGridDyPack >> (2 * m)) & 3u) - 1;
                lx -= dx;
                ly -= dy;
                cell -= (long long)dx + (long long)dy * W;
                if ((unsigned)lx >= (unsigned)kPathWin || (unsigned)ly >= (unsigned)kPathWin) break;
            }
            cx = x0 + lx;
            cy = y0 + ly;
            if (state == 0 && (cx < 0 || cx >= W || cy < 0 || cy >= H)) state = 2;
        }
        state = __shfl_sync(kFull, state, 0);
        cx = __shfl_sync(kFull, cx, 0);
        cy = __shfl_sync(kFull, cy, 0);
        len = __shfl_sync(kFull, len, 0);
        __syncwarp();  // the window is rewritten next
    }
    capped = __shfl_sync(kFull, (int)cp, 0) != 0;
    return state == 1 ? len : 0;
}

// walk_path for grids, by a whole warp (same arena protocol and statuses).
static __device__ void walk_grid_path(const InstDesc& d, unsigned long long* win, unsigned long long* arena,
                               unsigned long long arena_words, unsigned long long* arena_used, bool own_arena,
                               int lane, unsigned long long base_off) {
    InstCtl* ctl = d.ctl;
    const uint64_t limit = (uint64_t)ctl->best + 2;
    bool capped = false;
    if (own_arena) {
        const uint64_t len = walk_grid_warp(d, win, arena, arena_words, limit, lane, capped);
        if (lane != 0) return;
        if (!len || capped) {  // the host retries with room for best + 1 states
            ctl->status = ST_PATH_CAP;
            ctl->path_len = 0;
            return;
        }
        ctl->path_len = (uint32_t)len;
        ctl->path_off = base_off;
        atomicAdd(arena_used, (unsigned long long)len);
        return;
    }
    const uint64_t len = walk_grid_warp(d, win, nullptr, 0, limit, lane, capped);
    if (!len) {
        if (lane == 0) {
            ctl->status = ST_PATH_CAP;
            ctl->path_len = 0;
        }
        return;
    }
    unsigned long long off = 0;
    if (lane == 0) {
        off = atomicAdd(arena_used, (unsigned long long)len);
        ctl->path_len = (uint32_t)len;
    }
    off = __shfl_sync(kFull, off, 0);
    if (off + len > arena_words) {
        if (lane == 0) ctl->status = ST_PATH_CAP;
        return;
    }
    if (lane == 0) ctl->path_off = off;
    walk_grid_warp(d, win, arena + off, len, limit, lane, capped);
}

// One warp per finished instance: grids walk windows (walk_grid_path),
// puzzles walk on lane 0.  Blocks of kPathWarps warps, a window of shared
// memory per warp.  With `offs` (n + 1 prefix offsets) instance i owns arena
// words [offs[i], offs[i+1]) and writes as it walks; otherwise a launch of
// one owns the arena and larger launches reserve slices with an atomic.
static __global__ void __launch_bounds__(kPathWarps * 32)
    path_kernel(const InstDesc* insts, uint32_t n, unsigned long long* arena, unsigned long long arena_words,
                unsigned long long* arena_used, const unsigned long long* offs) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t i = blockIdx.x * kPathWarps + warp;
    if (i >= n) return;  // warp-uniform from here on: every lane reads the same instance
    const InstDesc& d = insts[i];
    if (d.ctl->life != LIFE_DONE || d.ctl->status != ST_OK) return;
    const bool own = offs || n == 1;
    const unsigned long long base = offs ? offs[i] : 0ull;
    unsigned long long* a = arena + base;
    const unsigned long long words = offs ? offs[i + 1] - base : arena_words;
    if (d.kind == KIND_GRID) {
        unsigned long long* win = reinterpret_cast<unsigned long long*>(g_dyn_smem) + warp * kPathWin * kPathWin;
        walk_grid_path(d, win, a, words, arena_used, own, lane, base);
        return;
    }
    if (lane != 0) return;
    switch (d.kind) {
        case KIND_SLIDING3: {
            SlidingDom<3>::Ctx c;
            sliding_ctx_min<3>(c, d);
            walk_path<SlidingDom<3>>(d, c, a, words, arena_used, own, base);
            break;
        }
        case KIND_SLIDING4: {
            SlidingDom<4>::Ctx c;
            sliding_ctx_min<4>(c, d);
            walk_path<SlidingDom<4>>(d, c, a, words, arena_used, own, base);
            break;
        }
        case KIND_SLIDING5: {
            SlidingDom<5>::Ctx c;
            sliding_ctx_min<5>(c, d);
            walk_path<SlidingDom<5>>(d, c, a, words, arena_used, own, base);
            break;
        }
        default:
            break;
    }
}

}  // namespace gastar
