// Generic problem plugins: the reference's plugin API (functional_types.h:6-10)
// on the GA* engine.  A plugin is a state type T (trivially copyable, at most
// 32 bytes, equal states with equal bytes -- the reference's padding fill,
// a_star_sliding_puzzle.h:76-81), a device successor function
//   void gen(const T& src, T& dst, bool& exists, uint32_t& cost, unsigned char i)
// for i < max_neighbours, and a device heuristic uint32_t h(const T&).
//
// States are stored as their bytes in KW = ceil(sizeof(T)/8) words.  The
// duplicate-detection table claims a slot with a CAS on a separate state word
// (so any byte pattern is a valid key) and records parents by slot index,
// since a plugin has no inverse moves: the path is rebuilt by following slot
// indices, like the reference's `prev` field (a_star.h:20-39, 132-135).
#pragma once

#include <cstring>

#include "search.cuh"

namespace gastar {

template <int KW> struct PlainKey {
    uint64_t w[KW];
    __device__ __forceinline__ bool operator==(const PlainKey& o) const {
#pragma unroll
        for (int j = 0; j < KW; ++j)
            if (w[j] != o.w[j]) return false;
        return true;
    }
};

template <int KW> __device__ __forceinline__ uint64_t hash_words(const PlainKey<KW>& k) {
    uint64_t h = 0x9e3779b97f4a7c15ull;
#pragma unroll
    for (int j = 0; j < KW; ++j) h = mix64(h ^ k.w[j]);
    return h;
}

// Slot = {state, key words, value}; state is empty (all ones), busy (all
// ones - 1) or a 62-bit tag of the key's hash once the key is written.
template <int KW> struct HashTabLock {
    static constexpr int SW = 2 + KW;
    unsigned long long* s;
    uint64_t mask;
    uint32_t max_probe;
};
constexpr uint64_t kBusy = ~0ull - 1;

template <int KW>
__device__ __forceinline__ bool lock_wait(const unsigned long long* st, uint64_t& v) {
    for (uint32_t spin = 0; v == kBusy; ++spin) {  // another thread is writing the key
        if (spin > (1u << 22)) return false;
        __nanosleep(32);
        v = __ldcg(st);
    }
    __threadfence();  // the key words written before the tag are visible now
    return true;
}

// Returns 1 claimed, 0 found, -1 full (or a writer that never finished).
template <int KW>
__device__ int lock_claim(const HashTabLock<KW>& t, const PlainKey<KW>& key, uint64_t& idx) {
    const uint64_t h = hash_words(key), tag = h >> 2;
    for (uint32_t p = 0; p < t.max_probe; ++p) {
        const uint64_t i = (h + p) & t.mask;
        unsigned long long* ss = t.s + i * HashTabLock<KW>::SW;
        uint64_t v = __ldcg(ss);
        if (v == kEmpty) {
            v = atomicCAS(ss, kEmpty, kBusy);
            if (v == kEmpty) {
#pragma unroll
                for (int j = 0; j < KW; ++j) __stcg(ss + 1 + j, key.w[j]);
                __threadfence();
                atomicExch(ss, tag);
                idx = i;
                return 1;
            }
        }
        if (!lock_wait<KW>(ss, v)) return -1;
        if (v != tag) continue;
        bool eq = true;
#pragma unroll
        for (int j = 0; j < KW; ++j) eq = eq && __ldcg(ss + 1 + j) == key.w[j];
        if (eq) {
            idx = i;
            return 0;
        }
    }
    return -1;
}

template <int KW>
__device__ uint64_t lock_get(const HashTabLock<KW>& t, const PlainKey<KW>& key, uint64_t& idx) {
    const uint64_t h = hash_words(key), tag = h >> 2;
    for (uint32_t p = 0; p < t.max_probe; ++p) {
        const uint64_t i = (h + p) & t.mask;
        const unsigned long long* ss = t.s + i * HashTabLock<KW>::SW;
        uint64_t v = __ldcg(ss);
        if (v == kEmpty) return kEmpty;
        if (!lock_wait<KW>(ss, v)) return kEmpty;
        if (v != tag) continue;
        bool eq = true;
#pragma unroll
        for (int j = 0; j < KW; ++j) eq = eq && __ldcg(ss + 1 + j) == key.w[j];
        if (eq) {
            idx = i;
            return __ldcg(ss + 1 + KW);
        }
    }
    return kEmpty;
}

template <typename T> constexpr int words_of() { return (int)((sizeof(T) + 7) / 8); }

template <typename T, unsigned char MAXN_,
          void (*GEN)(const T&, T&, bool&, uint32_t&, unsigned char), uint32_t (*HEUR)(const T&)>
struct PluginDom {
    static_assert(sizeof(T) <= 32, "plugin states are limited to 32 bytes");
    static constexpr int KW = words_of<T>();
    static constexpr int MAXN = MAXN_;
    static constexpr bool kDense = false;
    static constexpr uint32_t kRootCode = 0xffffffffu;
    static constexpr bool kParentBySlot = true;  // no inverse moves: parents by table slot
    struct Look {};                              // the own-slot lookup precedes the probes
    using KeyT = PlainKey<KW>;
    using Tab = HashTabLock<KW>;
    using Pre = int;

    struct Ctx {
        KeyT goal, start;
        uint32_t f0;
    };

    static __device__ __forceinline__ KeyT to_key(const T& t) {
        KeyT k;
#pragma unroll
        for (int j = 0; j < KW; ++j) k.w[j] = 0;
        memcpy(k.w, &t, sizeof(T));
        return k;
    }
    static __device__ __forceinline__ T from_key(const KeyT& k) {
        alignas(T) unsigned char buf[sizeof(T)];
        memcpy(buf, k.w, sizeof(T));
        return *reinterpret_cast<const T*>(buf);
    }
    static __device__ __forceinline__ KeyT desc_key(const uint64_t* lo2, const uint64_t* hi2) {
        KeyT k;
#pragma unroll
        for (int j = 0; j < KW; ++j) k.w[j] = j < 2 ? lo2[j] : hi2[j - 2];
        return k;
    }
    static __device__ __forceinline__ KeyT key_of(const Entry<KW>& e) {
        KeyT k;
#pragma unroll
        for (int j = 0; j < KW; ++j) k.w[j] = e.k[j];
        return k;
    }
    static __device__ __forceinline__ void set_key(Entry<KW>& e, const KeyT& k) {
#pragma unroll
        for (int j = 0; j < KW; ++j) e.k[j] = k.w[j];
    }

    static __device__ void load(Ctx& c, const InstDesc& d) {
        if (threadIdx.x == 0) {
            const uint64_t s2[2] = {d.start0, d.start1}, g2[2] = {d.goal0, d.goal1};
            c.start = desc_key(s2, d.start_hi);
            c.goal = desc_key(g2, d.goal_hi);
            c.f0 = HEUR(from_key(c.start));
        }
        __syncthreads();
    }
    static __device__ __forceinline__ uint32_t start_f(const Ctx& c, const InstDesc&) { return c.f0; }
    static __device__ __forceinline__ Tab make_tab(const InstDesc& d) {
        Tab t;
        t.s = d.table;
        t.mask = d.table_mask;
        t.max_probe = d.max_probe;
        return t;
    }
    static __device__ __forceinline__ uint64_t get(const Tab& t, const KeyT& k) {
        uint64_t i;
        return lock_get<KW>(t, k, i);
    }
    static __device__ __forceinline__ uint64_t get_self(const Tab& t, const KeyT& k, uint32_t& self) {
        uint64_t i = 0;
        const uint64_t v = lock_get<KW>(t, k, i);
        self = (uint32_t)i;
        return v;
    }
    static __device__ __forceinline__ uint32_t code(int, uint32_t self) { return self; }
    static __device__ __forceinline__ int insert(const Tab& t, const KeyT& k, uint64_t v, uint64_t& old,
                                                 uint64_t& slot) {
        uint64_t i;
        const int r = lock_claim<KW>(t, k, i);
        if (r < 0) return r;
        old = atomicMin(t.s + i * Tab::SW + 1 + KW, v);
        slot = i;
        return r;
    }
    static __device__ __forceinline__ int claim_first(const Tab& t, const KeyT& k, uint64_t, uint64_t& slot,
                                                      uint64_t&) {
        const int r = lock_claim<KW>(t, k, slot);
        return r < 0 ? r : kClNeedMin | r;
    }
    static __device__ __forceinline__ int claim_probe(const Tab&, const KeyT&, uint64_t, uint64_t&, uint64_t&) {
        return -1;
    }
    static __device__ __forceinline__ uint64_t min_at(const Tab& t, uint64_t slot, const KeyT&, uint64_t v,
                                                      uint64_t) {
        return atomicMin(t.s + slot * Tab::SW + 1 + KW, v);
    }
    static __device__ __forceinline__ bool is_goal(const Ctx& c, const KeyT& k) { return k == c.goal; }
    static __device__ __forceinline__ bool is_start(const Ctx& c, const KeyT& k) { return k == c.start; }
    static __device__ __forceinline__ Pre prepare(const Ctx&, const KeyT&) { return 0; }
    static __device__ __forceinline__ bool succ(const Ctx&, const KeyT& k, Pre, int m, uint32_t, uint32_t g,
                                                uint32_t, KeyT& nk, uint32_t& ng, uint32_t& nh) {
        const T src = from_key(k);
        T dst = src;
        bool ex = false;
        uint32_t cost = 0;
        GEN(src, dst, ex, cost, (unsigned char)m);
        if (!ex) return false;
        nk = to_key(dst);
        ng = g + cost;
        nh = HEUR(dst);
        return true;
    }
    static __device__ __forceinline__ KeyT parent(const Ctx&, const Tab& t, const KeyT&, uint32_t code) {
        KeyT k;
        const unsigned long long* ss = t.s + (uint64_t)code * Tab::SW;
#pragma unroll
        for (int j = 0; j < KW; ++j) k.w[j] = __ldcg(ss + 1 + j);
        return k;
    }
};

// One plugin instance on every block of the launch (cooperative when the
// team has more than one block).
template <class D> __global__ void __launch_bounds__(256, 1) plugin_search_kernel(LaunchParams P) {
    __shared__ CtaShared sm;
    __shared__ typename D::Ctx ctx;
    if (threadIdx.x == 0) sm.desc = P.insts[0];
    __syncthreads();
    run_instance<D>(P, sm.desc, sm, ctx, TeamRef{P.team_ctas, P.team_ctas > 1 ? blockIdx.x : 0u, P.team, P.stage});
}

template <class D>
__global__ void plugin_path_kernel(const InstDesc* insts, unsigned long long* arena,
                                   unsigned long long arena_words, unsigned long long* used) {
    if (blockIdx.x || threadIdx.x) return;
    const InstDesc& d = insts[0];
    if (d.ctl->life != LIFE_DONE || d.ctl->status != ST_OK) return;
    typename D::Ctx c;
    const uint64_t s2[2] = {d.start0, d.start1}, g2[2] = {d.goal0, d.goal1};
    c.start = D::desc_key(s2, d.start_hi);
    c.goal = D::desc_key(g2, d.goal_hi);
    // Same two-pass walk as walk_path, keys of KW words.
    InstCtl* ctl = d.ctl;
    const typename D::Tab tab = D::make_tab(d);
    const uint64_t limit = (uint64_t)ctl->best + 2;
    uint64_t len = 1;
    for (typename D::KeyT k = c.goal; !D::is_start(c, k); ++len) {
        const uint64_t v = D::get(tab, k);
        if (v == kEmpty || (uint32_t)v == D::kRootCode || len > limit) {
            ctl->status = ST_PATH_CAP;
            ctl->path_len = 0;
            return;
        }
        k = D::parent(c, tab, k, (uint32_t)v);
    }
    const unsigned long long words = len * D::KW;
    const unsigned long long off = atomicAdd(used, words);
    ctl->path_len = (uint32_t)len;
    if (off + words > arena_words) {
        ctl->status = ST_PATH_CAP;
        return;
    }
    ctl->path_off = off;
    typename D::KeyT k = c.goal;
    for (uint64_t i = 0; i < len; ++i) {
        for (int j = 0; j < D::KW; ++j) arena[off + i * D::KW + j] = k.w[j];
        if (i + 1 < len) k = D::parent(c, tab, k, (uint32_t)D::get(tab, k));
    }
}

}  // namespace gastar
