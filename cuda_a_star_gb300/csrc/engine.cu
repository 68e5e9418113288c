// Host runtime and C ABI of the GA* engine (libgastar.so).
//
// Plain mode  : one instance per launch; a team of thread blocks (cooperative
//               launch, device-side barriers) runs the whole search without a
//               host round trip.  Replaces a_star() (a_star.h:223-282).
// Batch mode  : many instances in one persistent launch, one block per
//               instance at a time, per-instance table/heap partitions.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gastar.h"
#include "engine_internal.h"
#include "search.cuh"

namespace gastar {

// Launch block of a plain solve (one device allocation, one upload):
// descriptor | control block | work counter | path counter | team control.
// The upload ends after the team control's first line (barrier counter,
// abort flag): the team's first block clears the cut slots itself.
constexpr size_t kLbAlign = 128;
constexpr size_t lb_round(size_t x) { return (x + kLbAlign - 1) / kLbAlign * kLbAlign; }
constexpr size_t kLbDesc = 0;
constexpr size_t kLbCtl = lb_round(sizeof(InstDesc));
constexpr size_t kLbNext = kLbCtl + lb_round(sizeof(InstCtl));
constexpr size_t kLbUsed = kLbNext + kLbAlign;
constexpr size_t kLbTeam = kLbUsed + kLbAlign;
constexpr size_t kLbBytes = kLbTeam + lb_round(sizeof(TeamCtl));
constexpr size_t kLbUpload = kLbTeam + kLbAlign;
constexpr uint64_t kPathPrefixWords = 1024;   // path words read back with the control block
constexpr uint64_t kPathArenaWords = 1 << 16;  // first path arena of a puzzle solve

thread_local std::string g_last_error;

void set_error(const std::string& s) { g_last_error = s; }

bool cuda_ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    set_error(std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
    return false;
}

#define GA_CUDA(call)                                  \
    do {                                               \
        if (!cuda_ok((call), #call)) return GASTAR_CUDA_ERROR; \
    } while (0)

void DevBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
}

bool DevBuf::ensure(size_t bytes) {
    fresh = false;
    if (bytes <= n) return true;
    release();
    fresh = true;
    size_t want = bytes < 256 ? 256 : bytes;
    if (!cuda_ok(cudaMalloc(&p, want), "cudaMalloc")) {
        p = nullptr;
        return false;
    }
    n = want;
    return true;
}

template <uint32_t K, int T = 256> const void* kernel_ptr() {
    return reinterpret_cast<const void*>(&search_kernel<K, T>);
}

const void* search_kernel_for(uint32_t kinds, uint32_t threads) {
    if (threads > 256) return kernel_ptr<kKindsAll, 512>();  // 9..16 warps: all kinds
    switch (kinds) {
        case kind_bit(KIND_SLIDING3): return kernel_ptr<kind_bit(KIND_SLIDING3)>();
        case kind_bit(KIND_SLIDING4): return kernel_ptr<kind_bit(KIND_SLIDING4)>();
        case kind_bit(KIND_SLIDING5): return kernel_ptr<kind_bit(KIND_SLIDING5)>();
        case kind_bit(KIND_GRID): return kernel_ptr<kind_bit(KIND_GRID)>();
        default: return kernel_ptr<kKindsAll>();
    }
}

uint32_t entry_bytes(uint32_t kind) { return kind == KIND_SLIDING5 ? 32u : 16u; }
uint32_t max_neighbours(uint32_t kind) { return kind == KIND_GRID ? 8u : 4u; }
uint32_t key_words(uint32_t kind) { return kind == KIND_SLIDING5 ? 2u : 1u; }

size_t block_smem_bytes(uint32_t kinds, uint32_t warps, uint32_t ew, bool multi, uint32_t heap_snodes,
                        bool buckets) {
    // Two stage buffers (one-block teams) + per warp: shared-memory heap
    // nodes and the bucket push scratch.
    size_t best = 0;
    for (uint32_t k = 0; k < 4; ++k)
        if (kinds & kind_bit(k)) {
            const size_t stage = multi ? 0 : 2 * stage_entries_per_buffer(warps, ew, max_neighbours(k)) * entry_bytes(k);
            const size_t per_warp = (size_t)(heap_snodes - 1) * 32 * entry_bytes(k) + (buckets ? 256 : 0);
            best = std::max(best, stage + ((size_t)warps * per_warp + 15) / 16 * 16);
        }
    return best;
}

uint32_t fit_heap_snodes(gastar_ctx* c, uint32_t kinds, uint32_t warps, uint32_t ew, bool multi, uint32_t threads,
                         int blocks_per_sm, size_t* smem, bool buckets) {
    *smem = block_smem_bytes(kinds, warps, ew, multi, kHeapSmemNodes, buckets);
    if (blocks_per_sm <= 0) return kHeapSmemNodes;
    const size_t reserve = 4096;  // static shared memory + per-block system share
    size_t budget = c->smem_per_sm / (size_t)blocks_per_sm;
    budget = budget > reserve ? std::min(budget - reserve, c->smem_optin - reserve) : 0;
    const size_t base = block_smem_bytes(kinds, warps, ew, multi, 1, buckets);
    const size_t node = block_smem_bytes(kinds, warps, ew, multi, 2, buckets) - base;  // one node in every warp
    if (!node || budget <= base + (kHeapSmemNodes - 1) * node) return kHeapSmemNodes;
    const uint32_t cand = (uint32_t)std::min<uint64_t>(1 + (budget - base) / node, kHeapSmemNodesMax);
    const size_t s2 = block_smem_bytes(kinds, warps, ew, multi, cand, buckets);
    if (occupancy_blocks(c, kinds, threads, s2) < blocks_per_sm) return kHeapSmemNodes;
    *smem = s2;
    return cand;
}

int occupancy_blocks(gastar_ctx* /*c: the current device's context*/, uint32_t kinds, uint32_t threads,
                     size_t smem) {
    const void* f = search_kernel_for(kinds, threads);
    if (smem > kSmemNoOptIn)
        if (!cuda_ok(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                     "cudaFuncSetAttribute"))
            return 0;
    int nb = 0;
    if (!cuda_ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, f, (int)threads, smem),
                 "cudaOccupancyMaxActiveBlocksPerMultiprocessor"))
        return 0;
    return nb;
}

int launch_search(gastar_ctx* /*c: the current device's context*/, uint32_t kinds, const LaunchParams& P,
                  uint32_t blocks, uint32_t threads, size_t smem, cudaStream_t st) {
    const void* f = search_kernel_for(kinds, threads);
    if (smem > kSmemNoOptIn)
        GA_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    LaunchParams p = P;
    void* args[] = {&p};
    // Blocks that wait on each other (multi-block teams) need a cooperative
    // launch, which guarantees they are resident together.
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(blocks);
    lc.blockDim = dim3(threads);
    lc.dynamicSmemBytes = smem;
    lc.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = (P.team_ctas > 1 || P.n_heavy > 0) ? 1 : 0;
    lc.attrs = attr;
    lc.numAttrs = 1;
    GA_CUDA(cudaLaunchKernelExC(&lc, f, args));
    return GASTAR_OK;
}

int launch_paths(const InstDesc* d_insts, uint32_t n, unsigned long long* arena,
                 unsigned long long arena_words, unsigned long long* used, cudaStream_t st,
                 const unsigned long long* offs) {
    const size_t smem = (size_t)kPathWarps * kPathWin * kPathWin * sizeof(unsigned long long);
    path_kernel<<<(n + kPathWarps - 1) / kPathWarps, kPathWarps * 32, smem, st>>>(d_insts, n, arena, arena_words,
                                                                                 used, offs);
    GA_CUDA(cudaGetLastError());
    return GASTAR_OK;
}

// ---------------------------------------------------------------------------
// Problem encoding on the host.
// ---------------------------------------------------------------------------
bool valid_board(uint32_t n, const uint8_t* b) {
    if (n < 3 || n > 5 || !b) return false;
    uint32_t seen = 0;
    for (uint32_t i = 0; i < n * n; ++i) {
        if (b[i] >= n * n || (seen >> b[i]) & 1u) return false;
        seen |= 1u << b[i];
    }
    return true;
}

void pack_board(uint32_t n, const uint8_t* b, uint64_t& lo, uint64_t& hi) {
    const uint32_t B = n <= 4 ? 4 : 5;
    unsigned __int128 k = 0;
    for (uint32_t i = 0; i < n * n; ++i) k |= (unsigned __int128)b[i] << (B * i);
    lo = (uint64_t)k;
    hi = (uint64_t)(k >> 64);
}

void unpack_board(uint32_t n, uint64_t lo, uint64_t hi, uint8_t* b) {
    const uint32_t B = n <= 4 ? 4 : 5;
    const unsigned __int128 k = ((unsigned __int128)hi << 64) | lo;
    for (uint32_t i = 0; i < n * n; ++i) b[i] = (uint8_t)((k >> (B * i)) & ((1u << B) - 1));
}

uint32_t sliding_h(uint32_t n, const uint8_t* b, const uint8_t* goal, uint32_t heuristic) {
    if (heuristic == GASTAR_H_ZERO) return 0;
    int gr[32], gc[32];
    for (uint32_t i = 0; i < n * n; ++i) {
        gr[goal[i]] = (int)(i / n);
        gc[goal[i]] = (int)(i % n);
    }
    uint32_t s = 0;
    for (uint32_t i = 0; i < n * n; ++i) {
        if (b[i] == 0 && heuristic != GASTAR_H_REFERENCE) continue;
        s += (uint32_t)(std::abs(gr[b[i]] - (int)(i / n)) + std::abs(gc[b[i]] - (int)(i % n)));
    }
    return s;
}

bool sliding_solvable(uint32_t n, const uint8_t* s, const uint8_t* g) {
    auto inv = [n](const uint8_t* b) {
        uint32_t c = 0, blank = 0;
        for (uint32_t i = 0; i < n * n; ++i) {
            if (!b[i]) {
                blank = i;
                continue;
            }
            for (uint32_t j = i + 1; j < n * n; ++j)
                if (b[j] && b[j] < b[i]) ++c;
        }
        if ((n & 1) == 0) c += blank / n;
        return c & 1u;
    };
    return inv(s) == inv(g);
}

uint32_t grid_h(uint32_t x, uint32_t y, uint32_t tx, uint32_t ty, uint32_t minw, uint32_t heuristic) {
    const uint32_t ax = x > tx ? x - tx : tx - x, ay = y > ty ? y - ty : ty - y;
    if (heuristic == GASTAR_H_REFERENCE) return ax + ay;
    if (heuristic == GASTAR_H_ZERO) return 0;
    return std::max(ax, ay) * minw;
}

uint64_t next_pow2(uint64_t v) {
    uint64_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

}  // namespace gastar

using namespace gastar;

// ---------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------
extern "C" {

int gastar_version(void) { return 100; }

const char* gastar_last_error(void) { return g_last_error.c_str(); }

const char* gastar_status_name(int s) {
    static const char* names[] = {"OK", "NO_PATH", "BUDGET", "TIMEOUT", "HEAP_FULL", "TABLE_FULL",
                                  "PATH_CAP", "BARRIER_TIMEOUT", "BAD_INPUT", "CUDA_ERROR",
                                  "NO_DEVICE", "PENDING", "OUT_OF_MEMORY", "COST_RANGE"};
    if (s < 0 || s >= (int)(sizeof(names) / sizeof(names[0]))) return "UNKNOWN";
    return names[s];
}

void gastar_config_default(gastar_config* cfg) {
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->num_queues = 4096;
    cfg->heuristic = GASTAR_H_ADMISSIBLE;
    cfg->moves = GASTAR_MOVES_STANDARD;
    cfg->expansion_width = 0;  // auto
    cfg->warps_per_block = 0;  // auto
    cfg->load_factor = 0.75f;
    cfg->regrow = 1;
}

gastar_ctx* gastar_create(int device) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        set_error("no CUDA device");
        return nullptr;
    }
    if (device < 0 && cudaGetDevice(&device) != cudaSuccess) device = 0;
    if (device >= count) {
        set_error("device index out of range");
        return nullptr;
    }
    if (!cuda_ok(cudaSetDevice(device), "cudaSetDevice")) return nullptr;
    auto* c = new gastar_ctx();
    c->device = device;
    cudaDeviceProp prop;
    if (!cuda_ok(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties")) {
        delete c;
        return nullptr;
    }
    c->sms = prop.multiProcessorCount;
    c->mem_total = prop.totalGlobalMem;
    std::snprintf(c->name, sizeof(c->name), "%s", prop.name);
    c->coop = prop.cooperativeLaunch;
    c->smem_per_sm = prop.sharedMemPerMultiprocessor;
    c->smem_optin = prop.sharedMemPerBlockOptin;
    {
        int pageable = 0, host_tables = 0;
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device);
        cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device);
        c->can_read_host = pageable == 1 && host_tables == 1;
        // Grid uploads: staged by default; GASTAR_UPLOAD=inplace (where the
        // GPU reads pageable host memory) or copy choose the others.
        const char* u = std::getenv("GASTAR_UPLOAD");
        c->upload_mode = u && !std::strcmp(u, "copy") ? 0 : u && !std::strcmp(u, "inplace") && c->can_read_host ? 1 : 2;
    }
    if (!cuda_ok(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !cuda_ok(cudaEventCreate(&c->e0), "cudaEventCreate") ||
        !cuda_ok(cudaEventCreate(&c->e1), "cudaEventCreate") ||
        !cuda_ok(cudaMallocHost(&c->h_ctl, sizeof(InstCtl)), "cudaMallocHost") ||
        !cuda_ok(cudaMallocHost(&c->h_launch, kLbBytes), "cudaMallocHost") ||
        !cuda_ok(cudaMallocHost(reinterpret_cast<void**>(&c->h_path), kPathPrefixWords * 8), "cudaMallocHost")) {
        delete c;
        return nullptr;
    }
    return c;
}

void gastar_destroy(gastar_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->table.release();
    c->dense.release();
    c->touched.release();
    c->buckets.release();
    c->heaps.release();
    c->hdr.release();
    c->stage.release();
    c->launch.release();
    c->path.release();
    c->misc.release();
    c->weights.release();
    destroy_stager(c->stager);
    if (c->h_ctl) cudaFreeHost(c->h_ctl);
    if (c->h_launch) cudaFreeHost(c->h_launch);
    if (c->h_path) cudaFreeHost(c->h_path);
    if (c->e0) cudaEventDestroy(c->e0);
    if (c->e1) cudaEventDestroy(c->e1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int gastar_device_info(gastar_ctx* c, int* sm_count, uint64_t* mem_bytes, char* name, size_t name_len) {
    if (!c) return GASTAR_BAD_INPUT;
    if (sm_count) *sm_count = c->sms;
    if (mem_bytes) *mem_bytes = c->mem_total;
    if (name && name_len) std::snprintf(name, name_len, "%s", c->name);
    return GASTAR_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Plain engine
// ---------------------------------------------------------------------------
namespace gastar {

static void fill_result(gastar_result* out, const InstCtl& c) {
    out->status = (int32_t)c.status;
    out->cost = c.status == ST_OK || c.status == ST_PATH_CAP ? c.best : 0;
    out->path_len = c.path_len;
    out->iterations = c.iterations;
    out->expansions = c.expansions;
    out->generated = c.generated;
    out->pushes = c.pushes;
    out->stale = c.stale;
    out->table_used = c.table_used;
}

struct AttemptStats {
    float kernel_ms = 0;
    uint32_t launches = 0;
    uint64_t h2d = 0, d2h = 0;
};

// Runs the search (+ path rebuild) once with the given capacities.
static int plain_attempt(gastar_ctx* c, const PlainProblem& pp, const gastar_config& cfg,
                         uint32_t table_log2, uint64_t heap_entries, std::vector<uint64_t>* path_keys,
                         cudaStream_t st, InstCtl& ctl_out, AttemptStats& as) {
    const bool want_path = path_keys != nullptr;
    const uint32_t kinds = kind_bit(pp.kind);
    // Expansion width 0 = about 1024 warp-heaps per solve: wide enough pops
    // for large Q, enough heaps (warps) to keep the SMs busy for small Q.
    const uint32_t ew = cfg.expansion_width
                            ? std::min(32u, cfg.expansion_width)
                            : (uint32_t)std::min<uint64_t>(32, std::max<uint64_t>(8, (cfg.num_queues ? cfg.num_queues : 4096) / 1024));
    const uint64_t Q = cfg.num_queues ? cfg.num_queues : 4096;
    uint64_t heaps = (Q + ew - 1) / ew;
    // Warps per block 0 = 8 when that still gives at least half of the SMs a
    // block (fewer, larger blocks: fewer parties to the hand-offs), else 4.
    const uint32_t W = cfg.warps_per_block ? std::min(16u, cfg.warps_per_block)
                                           : ((heaps / 8 >= (uint64_t)c->sms / 2) ? 8u : 4u);
    const uint32_t threads = W * 32;
    uint64_t blocks = (heaps + W - 1) / W;
    const bool multi = blocks > 1;
    // Widening: a puzzle search with the automatic width that passes
    // kWideAfter iterations is a hard one, whose iteration count the pops per
    // iteration set rather than its depth; from then on every warp-heap pops
    // twice as many (at most 32).  On the 64 15-puzzles of the plain
    // benchmark (Q = 16384) the four hardest took 150-359 iterations and ran
    // 1.3-1.4x faster with twice the pops, the rest at most ~90 iterations.
    const uint32_t ew_wide =
        multi && pp.kind != KIND_GRID && !cfg.expansion_width ? std::min(32u, 2 * ew) : ew;
    size_t smem = block_smem_bytes(kinds, W, ew, multi);
    const int nb = occupancy_blocks(c, kinds, threads, smem);
    if (nb <= 0) return GASTAR_CUDA_ERROR;
    uint64_t max_blocks = (uint64_t)nb * c->sms;
    if (cfg.max_blocks) max_blocks = std::min<uint64_t>(max_blocks, cfg.max_blocks);
    if (blocks > max_blocks) blocks = max_blocks;
    // The shared memory the co-resident blocks leave free holds the heaps' top
    // levels: pops and pushes then touch global nodes only deep down.
    const bool buckets = cfg.open_list == 1;
    const uint32_t snodes = fit_heap_snodes(c, kinds, W, ew, multi, threads,
                                            (int)((blocks + c->sms - 1) / c->sms), &smem, buckets);
    if (multi && !c->coop) {
        set_error("device does not support cooperative launch");
        return GASTAR_CUDA_ERROR;
    }
    heaps = blocks * W;
    const uint32_t maxn = max_neighbours(pp.kind);

    // Duplicate-detection table: a dense per-cell array for grids (cleared by
    // the kernel), a hash table for puzzles that stays allocated across solves
    // and is cleared slot by slot from the previous solve's claim list.
    const uint32_t ebytes = entry_bytes(pp.kind), kw = key_words(pp.kind);
    const uint32_t slot_words = kw == 1 ? 2 : 4;
    uint64_t table_words, mask = 0, limit = ~0ull, touched_cap = 0;
    DevBuf* tb;
    if (pp.kind == KIND_GRID) {
        table_words = (uint64_t)pp.W * pp.H;
        tb = &c->dense;
        if (!tb->ensure(table_words * 8)) return GASTAR_OUT_OF_MEMORY;
    } else {
        const uint64_t slots = 1ull << table_log2;
        table_words = slots * slot_words;
        mask = slots - 1;
        float lf = cfg.load_factor > 0.f ? cfg.load_factor : 0.75f;
        lf = std::min(0.95f, std::max(0.1f, lf));
        limit = (uint64_t)((double)slots * lf);
        // Claims stop within two iterations past the limit; every warp may
        // leave one chunk partly unused.
        touched_cap = limit + 2 * heaps * ew_wide * maxn + heaps * kTouchedChunk + 16;
        tb = &c->table;
        // A reallocated table, claim list or claim counter loses the record of
        // what the previous solve wrote: clear the whole table then.
        bool lost = false;
        if (!tb->ensure(table_words * 8)) return GASTAR_OUT_OF_MEMORY;
        lost |= tb->fresh;
        if (!c->touched.ensure(touched_cap * 4)) return GASTAR_OUT_OF_MEMORY;
        lost |= c->touched.fresh;
        if (!c->misc.ensure(64)) return GASTAR_OUT_OF_MEMORY;
        lost |= c->misc.fresh;
        touched_cap = c->touched.n / 4;
        if (lost || c->table_dirty) {
            GA_CUDA(cudaMemsetAsync(tb->p, 0xff, tb->n, st));
            GA_CUDA(cudaMemsetAsync(c->misc.p, 0, 8, st));  // claim-list length
            c->table_dirty = false;
        }
    }
    // Heaps: per warp-heap node capacity with headroom for uneven dealing.
    uint64_t per_heap = (heap_entries + heaps - 1) / heaps;
    uint64_t cap_nodes = std::max<uint64_t>(2 * snodes, (per_heap * 2 + 31) / 32);
    if (cap_nodes > 0x7fffffffull) return GASTAR_OUT_OF_MEMORY;
    const size_t heap_bytes = (size_t)heaps * (cap_nodes + 1) * 32 * ebytes;
    const size_t stage_bytes = multi ? team_stage_bytes((uint32_t)blocks, W, ew_wide, maxn, ebytes) : 16;

    if (!c->heaps.ensure(heap_bytes) || !c->hdr.ensure((size_t)heaps * 8) ||
        !c->stage.ensure(stage_bytes) || !c->launch.ensure(kLbBytes))
        return GASTAR_OUT_OF_MEMORY;
    char* const lb = static_cast<char*>(c->launch.p);
    // Bucket front: as many pages per warp as the heap has nodes.
    if (buckets && !c->buckets.ensure(bucket_area_bytes((uint32_t)heaps, (uint32_t)cap_nodes, ebytes)))
        return GASTAR_OUT_OF_MEMORY;

    InstDesc d;
    std::memset(&d, 0, sizeof(d));
    d.kind = pp.kind;
    d.heuristic = cfg.heuristic;
    d.moves = cfg.moves;
    d.n = pp.n;
    d.start0 = pp.start0;
    d.start1 = pp.start1;
    d.goal0 = pp.goal0;
    d.goal1 = pp.goal1;
    d.weights = pp.d_weights;
    d.W = pp.W;
    d.H = pp.H;
    d.minw = pp.minw;
    d.f0 = pp.f0;
    d.table = reinterpret_cast<unsigned long long*>(tb->p);
    d.table_words = table_words;
    d.table_mask = mask;
    d.table_limit = limit;
    d.max_probe = 4096;
    d.heaps = (uint32_t)heaps;
    d.heap_nodes = c->heaps.p;
    d.heap_hdr = reinterpret_cast<uint32_t*>(c->hdr.p);
    d.heap_cap = (uint32_t)cap_nodes;
    d.ew = ew;
    if (ew_wide > ew) {
        d.ew_wide = ew_wide;
        d.wide_after = kWideAfter;
    }
    d.max_exp = cfg.max_expansions;
    d.timeout_ns = (uint64_t)cfg.timeout_ms * 1000000ull;
    d.max_iter = cfg.max_iterations;
    d.delta = cfg.delta;
    d.ctl = reinterpret_cast<InstCtl*>(lb + kLbCtl);
    if (buckets) {
        d.bq_base = c->buckets.p;
        d.bq_pages = (uint32_t)cap_nodes;
    }
    if (pp.kind != KIND_GRID) {
        d.touched = reinterpret_cast<uint32_t*>(c->touched.p);
        d.touched_count = reinterpret_cast<unsigned long long*>(c->misc.p);
        d.touched_cap = touched_cap;
        d.prev_slot_words = c->prev_slot_words;
    }
    // Descriptor, zeroed control block, team control and counters: one copy.
    char* const hl = static_cast<char*>(c->h_launch);
    std::memset(hl, 0, kLbBytes);
    std::memcpy(hl + kLbDesc, &d, sizeof(InstDesc));
    team_ctl_init(*reinterpret_cast<TeamCtl*>(hl + kLbTeam));

    LaunchParams P;
    std::memset(&P, 0, sizeof(P));
    P.insts = reinterpret_cast<const InstDesc*>(lb + kLbDesc);
    P.n_insts = 1;
    P.next = reinterpret_cast<uint32_t*>(lb + kLbNext);
    P.team_ctas = (uint32_t)blocks;
    P.heap_snodes = snodes;
    P.buckets = buckets ? 1u : 0u;
    P.team = reinterpret_cast<TeamCtl*>(lb + kLbTeam);
    P.stage = c->stage.p;
    P.barrier_timeout_ns = 2000000000ull;

    GA_CUDA(cudaMemcpyAsync(lb, hl, kLbUpload, cudaMemcpyHostToDevice, st));
    as.h2d += kLbUpload;
    GA_CUDA(cudaEventRecord(c->e0, st));
    int rc = launch_search(c, kinds, P, (uint32_t)blocks, threads, smem, st);
    if (rc != GASTAR_OK) return rc;
    ++as.launches;
    GA_CUDA(cudaEventRecord(c->e1, st));
    // The path rebuild follows on the stream (it checks the status itself);
    // the control block and the path's first words come back together.
    unsigned long long* const used = reinterpret_cast<unsigned long long*>(lb + kLbUsed);
    uint64_t prefix = 0;
    if (want_path) {
        const uint64_t arena_words =
            pp.kind == KIND_GRID ? (uint64_t)pp.W * pp.H + 2 : kPathArenaWords;  // a grid path visits a cell once
        if (!c->path.ensure(arena_words * 8 + 16)) return GASTAR_OUT_OF_MEMORY;
        rc = launch_paths(P.insts, 1, reinterpret_cast<unsigned long long*>(c->path.p), c->path.n / 8, used, st);
        if (rc != GASTAR_OK) return rc;
        ++as.launches;
        prefix = std::min<uint64_t>(kPathPrefixWords, c->path.n / 8);
        GA_CUDA(cudaMemcpyAsync(c->h_path, c->path.p, prefix * 8, cudaMemcpyDeviceToHost, st));
        as.d2h += prefix * 8;
    }
    GA_CUDA(cudaMemcpyAsync(c->h_ctl, lb + kLbCtl, sizeof(InstCtl), cudaMemcpyDeviceToHost, st));
    GA_CUDA(cudaStreamSynchronize(st));
    as.d2h += sizeof(InstCtl);
    if (pp.kind != KIND_GRID) {
        c->prev_slot_words = slot_words;
        // Reserved entries <= 1 + claims + one chunk per warp: beyond the
        // list's size some claims went unrecorded.
        if (1 + c->h_ctl->table_used + heaps * kTouchedChunk > touched_cap) c->table_dirty = true;
    }
    if (want_path && c->h_ctl->status == ST_PATH_CAP && c->h_ctl->best != kInf) {
        // Longer than the first arena: again with room for best + 1 states
        // (every step costs >= 1).
        const uint64_t words = ((uint64_t)c->h_ctl->best + 2) * kw;
        if (!c->path.ensure(words * 8 + 16)) return GASTAR_OUT_OF_MEMORY;
        InstCtl* hc = reinterpret_cast<InstCtl*>(hl + kLbCtl);
        *hc = *c->h_ctl;
        hc->status = ST_OK;
        hc->path_len = 0;
        GA_CUDA(cudaMemcpyAsync(lb + kLbCtl, hc, sizeof(InstCtl), cudaMemcpyHostToDevice, st));
        GA_CUDA(cudaMemsetAsync(used, 0, 8, st));
        rc = launch_paths(P.insts, 1, reinterpret_cast<unsigned long long*>(c->path.p), c->path.n / 8, used, st);
        if (rc != GASTAR_OK) return rc;
        ++as.launches;
        prefix = 0;
        GA_CUDA(cudaMemcpyAsync(c->h_ctl, lb + kLbCtl, sizeof(InstCtl), cudaMemcpyDeviceToHost, st));
        GA_CUDA(cudaStreamSynchronize(st));
        as.h2d += sizeof(InstCtl);
        as.d2h += sizeof(InstCtl);
    }
    if (want_path && c->h_ctl->status == ST_OK) {
        const uint64_t words = (uint64_t)c->h_ctl->path_len * kw, off = c->h_ctl->path_off;
        path_keys->resize(words);
        if (off + words <= prefix) {
            std::memcpy(path_keys->data(), c->h_path + off, words * 8);
        } else {
            GA_CUDA(cudaMemcpyAsync(path_keys->data(), reinterpret_cast<unsigned long long*>(c->path.p) + off,
                                    words * 8, cudaMemcpyDeviceToHost, st));
            GA_CUDA(cudaStreamSynchronize(st));
            as.d2h += words * 8;
        }
    }
    float ms = 0;
    GA_CUDA(cudaEventElapsedTime(&ms, c->e0, c->e1));
    as.kernel_ms += ms;
    ctl_out = *c->h_ctl;
    return GASTAR_OK;
}

int plain_solve(gastar_ctx* c, const PlainProblem& pp, const gastar_config* user_cfg,
                std::vector<uint64_t>* path_keys, gastar_result* out) {
    gastar_config cfg;
    if (user_cfg) cfg = *user_cfg;
    else gastar_config_default(&cfg);
    cudaStream_t st = cfg.stream ? (cudaStream_t)cfg.stream : c->stream;
    uint32_t table_log2 = cfg.table_log2;
    const uint32_t max_log2 = pp.kind == KIND_SLIDING5 ? 29 : 30;
    if (!table_log2) table_log2 = pp.kind == KIND_SLIDING3 ? 19 : 22;
    table_log2 = std::min(table_log2, max_log2);
    uint64_t heap_entries = cfg.heap_entries;
    if (!heap_entries)
        heap_entries = pp.kind == KIND_GRID ? std::max<uint64_t>(1 << 20, (uint64_t)pp.W * pp.H)
                                            : std::min<uint64_t>(1ull << table_log2, 1ull << 24);
    InstCtl ctl;
    AttemptStats as;
    uint32_t attempts = 0;
    for (;;) {
        ++attempts;
        int rc = plain_attempt(c, pp, cfg, table_log2, heap_entries, path_keys, st, ctl, as);
        if (rc != GASTAR_OK) return rc;
        if (!cfg.regrow) break;
        if (ctl.status == ST_TABLE_FULL && pp.kind != KIND_GRID && table_log2 < max_log2) {
            ++table_log2;
            continue;
        }
        if (ctl.status == ST_HEAP_FULL && heap_entries < (1ull << 32)) {
            heap_entries *= 2;
            continue;
        }
        break;
    }
    fill_result(out, ctl);
    out->kernel_ms = as.kernel_ms;
    out->attempts = attempts;
    out->launches = as.launches;
    out->h2d_bytes = as.h2d;
    out->d2h_bytes = as.d2h;
    c->launches += as.launches;
    return GASTAR_OK;
}

}  // namespace gastar

extern "C" {

int gastar_solve_sliding(gastar_ctx* c, uint32_t n, const uint8_t* start, const uint8_t* goal,
                         const gastar_config* cfg, uint8_t* path, uint32_t path_cap,
                         gastar_result* out) {
    auto t0 = std::chrono::steady_clock::now();
    if (!c || !out) return GASTAR_BAD_INPUT;
    std::memset(out, 0, sizeof(*out));
    if (!valid_board(n, start) || !valid_board(n, goal)) {
        set_error("sliding: boards must be permutations of 0..n*n-1 with n in 3..5");
        out->status = GASTAR_BAD_INPUT;
        return GASTAR_BAD_INPUT;
    }
    gastar_config dc;
    gastar_config_default(&dc);
    const gastar_config& cf = cfg ? *cfg : dc;
    if (cudaSetDevice(c->device) != cudaSuccess) return GASTAR_CUDA_ERROR;
    // The standard four-move puzzle splits into two parity classes; a goal in
    // the other class is unreachable, so there is no search to run.
    if (cf.moves == GASTAR_MOVES_STANDARD && !sliding_solvable(n, start, goal)) {
        out->status = GASTAR_NO_PATH;
        out->total_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
        return GASTAR_OK;
    }
    PlainProblem pp;
    std::memset(&pp, 0, sizeof(pp));
    pp.kind = n == 3 ? KIND_SLIDING3 : n == 4 ? KIND_SLIDING4 : KIND_SLIDING5;
    pp.n = n;
    pack_board(n, start, pp.start0, pp.start1);
    pack_board(n, goal, pp.goal0, pp.goal1);
    pp.f0 = sliding_h(n, start, goal, cf.heuristic);
    std::vector<uint64_t> keys;
    int rc = plain_solve(c, pp, cfg, path ? &keys : nullptr, out);
    if (rc != GASTAR_OK) {
        out->status = rc;
        return rc;
    }
    if (path && out->status == GASTAR_OK) {
        const uint32_t kw = key_words(pp.kind);
        if (out->path_len > path_cap) {
            out->status = GASTAR_PATH_CAP;
        } else {
            for (uint32_t i = 0; i < out->path_len; ++i) {  // stored goal-first
                const uint32_t j = out->path_len - 1 - i;
                unpack_board(n, keys[(size_t)j * kw], kw == 2 ? keys[(size_t)j * kw + 1] : 0,
                             path + (size_t)i * n * n);
            }
        }
    }
    out->total_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return GASTAR_OK;
}

static int solve_grid_impl(gastar_ctx* c, uint32_t w, uint32_t h, const uint8_t* d_weights,
                           uint32_t minw, uint32_t sx, uint32_t sy, uint32_t tx, uint32_t ty,
                           const gastar_config* cfg, uint32_t* path, uint32_t path_cap,
                           gastar_result* out, std::chrono::steady_clock::time_point t0) {
    gastar_config dc;
    gastar_config_default(&dc);
    const gastar_config& cf = cfg ? *cfg : dc;
    PlainProblem pp;
    std::memset(&pp, 0, sizeof(pp));
    pp.kind = KIND_GRID;
    pp.start0 = (uint64_t)sy * w + sx;
    pp.goal0 = (uint64_t)ty * w + tx;
    pp.d_weights = d_weights;
    pp.W = w;
    pp.H = h;
    pp.minw = minw;
    pp.f0 = grid_h(sx, sy, tx, ty, minw, cf.heuristic);
    std::vector<uint64_t> keys;
    int rc = plain_solve(c, pp, cfg, path ? &keys : nullptr, out);
    if (rc != GASTAR_OK) {
        out->status = rc;
        return rc;
    }
    if (path && out->status == GASTAR_OK) {
        if (out->path_len > path_cap) out->status = GASTAR_PATH_CAP;
        else
            for (uint32_t i = 0; i < out->path_len; ++i) path[i] = (uint32_t)keys[out->path_len - 1 - i];
    }
    out->total_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return GASTAR_OK;
}

static bool grid_args_ok(uint32_t w, uint32_t h, uint32_t sx, uint32_t sy, uint32_t tx, uint32_t ty) {
    return w && h && w <= 65535 && h <= 65535 && (uint64_t)w * h < (1ull << 32) && sx < w && sy < h &&
           tx < w && ty < h;
}

int gastar_solve_grid(gastar_ctx* c, uint32_t w, uint32_t h, const uint8_t* weights, uint32_t sx,
                      uint32_t sy, uint32_t tx, uint32_t ty, const gastar_config* cfg,
                      uint32_t* path, uint32_t path_cap, gastar_result* out) {
    auto t0 = std::chrono::steady_clock::now();
    if (!c || !out) return GASTAR_BAD_INPUT;
    std::memset(out, 0, sizeof(*out));
    if (!weights || !grid_args_ok(w, h, sx, sy, tx, ty)) {
        set_error("grid: bad dimensions or endpoints");
        out->status = GASTAR_BAD_INPUT;
        return GASTAR_BAD_INPUT;
    }
    if (cudaSetDevice(c->device) != cudaSuccess) return GASTAR_CUDA_ERROR;
    const size_t cells = (size_t)w * h;
    cudaStream_t st = (cfg && cfg->stream) ? (cudaStream_t)cfg->stream : c->stream;
    if (!c->weights.ensure(cells)) return GASTAR_OUT_OF_MEMORY;
    uint32_t minw = 255;
    int rc = upload_grid(c, reinterpret_cast<uint8_t*>(c->weights.p), weights, cells, st, &minw);
    if (rc != GASTAR_OK) return rc;
    rc = solve_grid_impl(c, w, h, reinterpret_cast<const uint8_t*>(c->weights.p), minw, sx, sy, tx,
                             ty, cfg, path, path_cap, out, t0);
    out->h2d_bytes += cells;
    return rc;
}

int gastar_solve_grid_device(gastar_ctx* c, uint32_t w, uint32_t h, const uint8_t* d_weights,
                             uint32_t sx, uint32_t sy, uint32_t tx, uint32_t ty,
                             const gastar_config* cfg, uint32_t* path, uint32_t path_cap,
                             gastar_result* out) {
    auto t0 = std::chrono::steady_clock::now();
    if (!c || !out) return GASTAR_BAD_INPUT;
    std::memset(out, 0, sizeof(*out));
    if (!d_weights || !grid_args_ok(w, h, sx, sy, tx, ty)) {
        set_error("grid: bad dimensions or endpoints");
        out->status = GASTAR_BAD_INPUT;
        return GASTAR_BAD_INPUT;
    }
    if (cudaSetDevice(c->device) != cudaSuccess) return GASTAR_CUDA_ERROR;
    cudaStream_t st = (cfg && cfg->stream) ? (cudaStream_t)cfg->stream : c->stream;
    uint32_t minw = 1;
    int rc = device_min_weight(c, d_weights, (uint64_t)w * h, st, &minw);
    if (rc != GASTAR_OK) return rc;
    return solve_grid_impl(c, w, h, d_weights, minw, sx, sy, tx, ty, cfg, path, path_cap, out, t0);
}

int gastar_grid_min_weight(gastar_ctx* c, uint32_t w, uint32_t h, const uint8_t* weights, uint32_t* minw,
                           int* upload_path) {
    if (!c || !weights || !minw || !w || !h) return GASTAR_BAD_INPUT;
    if (cudaSetDevice(c->device) != cudaSuccess) return GASTAR_CUDA_ERROR;
    const size_t cells = (size_t)w * h;
    if (!c->weights.ensure(cells)) return GASTAR_OUT_OF_MEMORY;
    if (upload_path) *upload_path = c->upload_mode;
    return upload_grid(c, reinterpret_cast<uint8_t*>(c->weights.p), weights, cells, c->stream, minw);
}

}  // extern "C"
