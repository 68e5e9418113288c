// Batched GA*: many puzzle and grid instances in one persistent launch.
//
// Each instance gets its own partition (duplicate-detection table + warp-heaps)
// sized from its class; a block takes instances from a work counter, largest
// first, and runs each to completion on its own (block-local barriers, stage
// buffer in shared memory).  The launch sequence (control reset, search,
// path rebuild, result copy) is captured once in a CUDA graph and replayed.
// The reference has no counterpart: its problem data sits in __constant__
// symbols, one instance per process (a_star_sliding_puzzle.h:125-128,
// a_star_pathfinding.h:72-81).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <numeric>
#include <vector>

#include "../../include/gastar.h"
#include "device_common.cuh"
#include "engine_internal.h"

namespace gastar {

__global__ void min_weight_kernel(const uint8_t* w, uint64_t cells, uint32_t* out) {
    uint32_t m = 255;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cells;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = w[i];
        if (v && v < m) m = v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(kFull, m, o));
    if ((threadIdx.x & 31) == 0) atomicMin(out, m);
}

int device_min_weight(gastar_ctx* c, const uint8_t* d_w, uint64_t cells, cudaStream_t st,
                      uint32_t* out) {
    if (!c->misc.ensure(64)) return GASTAR_OUT_OF_MEMORY;
    uint32_t* d = reinterpret_cast<uint32_t*>(c->misc.p) + 8;
    const uint32_t init = 255;
    if (!cuda_ok(cudaMemcpyAsync(d, &init, 4, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync"))
        return GASTAR_CUDA_ERROR;
    const uint64_t blocks = std::min<uint64_t>((cells + 255) / 256, (uint64_t)c->sms * 8);
    min_weight_kernel<<<(unsigned)std::max<uint64_t>(1, blocks), 256, 0, st>>>(d_w, cells, d);
    if (!cuda_ok(cudaGetLastError(), "min_weight_kernel")) return GASTAR_CUDA_ERROR;
    if (!cuda_ok(cudaMemcpyAsync(out, d, 4, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync") ||
        !cuda_ok(cudaStreamSynchronize(st), "cudaStreamSynchronize"))
        return GASTAR_CUDA_ERROR;
    return GASTAR_OK;
}

}  // namespace gastar

using namespace gastar;

struct BatchInst {
    uint32_t kind, n;
    uint64_t start0, start1, goal0, goal1;
    uint32_t W, H, minw, f0;
    std::vector<uint8_t> weights;  // grid
    uint64_t weights_off = 0;
    uint64_t est = 0;              // scheduling estimate (larger first)
};

struct gastar_batch {
    gastar_ctx* ctx = nullptr;
    gastar_batch_config cfg;
    std::vector<BatchInst> insts;
    bool uploaded = false;
    DevBuf arena, weights, descs, ctls, order, counters, paths;
    std::vector<InstDesc> h_desc;
    InstCtl* h_ctl = nullptr;               // pinned, n + 1 (last = arena counter)
    std::vector<unsigned long long> h_paths;
    uint64_t path_words = 0;
    uint32_t blocks = 0, threads = 0, n_sched = 0;
    size_t smem = 0;
    cudaGraphExec_t graph = nullptr;
    float kernel_ms = 0;
    uint64_t h2d = 0, d2h = 0, device_bytes = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
};

extern "C" {

void gastar_batch_config_default(gastar_batch_config* cfg) {
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->warps_per_block = 8;
    cfg->expansion_width = 32;
    cfg->load_factor = 0.75f;
    cfg->heuristic = GASTAR_H_ADMISSIBLE;
    cfg->moves = GASTAR_MOVES_STANDARD;
    cfg->use_graph = 1;
}

gastar_batch* gastar_batch_create(gastar_ctx* c, const gastar_batch_config* cfg) {
    if (!c) return nullptr;
    auto* b = new gastar_batch();
    b->ctx = c;
    if (cfg) b->cfg = *cfg;
    else gastar_batch_config_default(&b->cfg);
    if (!b->cfg.warps_per_block) b->cfg.warps_per_block = 8;
    if (!b->cfg.expansion_width) b->cfg.expansion_width = 32;
    if (b->cfg.load_factor <= 0.f) b->cfg.load_factor = 0.75f;
    b->cfg.warps_per_block = std::min(16u, b->cfg.warps_per_block);
    b->cfg.expansion_width = std::min(32u, b->cfg.expansion_width);
    cudaSetDevice(c->device);
    cudaEventCreate(&b->e0);
    cudaEventCreate(&b->e1);
    return b;
}

void gastar_batch_destroy(gastar_batch* b) {
    if (!b) return;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->arena.release();
    b->weights.release();
    b->descs.release();
    b->ctls.release();
    b->order.release();
    b->counters.release();
    b->paths.release();
    if (b->h_ctl) cudaFreeHost(b->h_ctl);
    if (b->e0) cudaEventDestroy(b->e0);
    if (b->e1) cudaEventDestroy(b->e1);
    delete b;
}

int gastar_batch_add_sliding(gastar_batch* b, uint32_t n, const uint8_t* start, const uint8_t* goal) {
    if (!b || b->uploaded) return -GASTAR_BAD_INPUT;
    if (!valid_board(n, start) || !valid_board(n, goal)) {
        set_error("sliding: boards must be permutations of 0..n*n-1 with n in 3..5");
        return -GASTAR_BAD_INPUT;
    }
    BatchInst in;
    in.kind = n == 3 ? KIND_SLIDING3 : n == 4 ? KIND_SLIDING4 : KIND_SLIDING5;
    in.n = n;
    pack_board(n, start, in.start0, in.start1);
    pack_board(n, goal, in.goal0, in.goal1);
    in.W = in.H = in.minw = 0;
    in.f0 = sliding_h(n, start, goal, b->cfg.heuristic);
    // Unsolvable (other parity class): mark with est = 0 and f0 = ~0.
    if (b->cfg.moves == GASTAR_MOVES_STANDARD && !sliding_solvable(n, start, goal)) in.f0 = kInf;
    in.est = (uint64_t)in.f0 * (n == 5 ? 4 : n == 4 ? 2 : 1);
    b->insts.push_back(std::move(in));
    return (int)b->insts.size() - 1;
}

int gastar_batch_add_grid(gastar_batch* b, uint32_t w, uint32_t h, const uint8_t* weights, uint32_t sx,
                          uint32_t sy, uint32_t tx, uint32_t ty) {
    if (!b || b->uploaded) return -GASTAR_BAD_INPUT;
    if (!weights || !w || !h || w > 65535 || h > 65535 || sx >= w || sy >= h || tx >= w || ty >= h) {
        set_error("grid: bad dimensions or endpoints");
        return -GASTAR_BAD_INPUT;
    }
    BatchInst in;
    in.kind = KIND_GRID;
    in.n = 0;
    in.W = w;
    in.H = h;
    in.start0 = (uint64_t)sy * w + sx;
    in.goal0 = (uint64_t)ty * w + tx;
    in.start1 = in.goal1 = 0;
    in.weights.assign(weights, weights + (size_t)w * h);
    uint32_t minw = 255;
    for (uint8_t v : in.weights)
        if (v && v < minw) minw = v;
    in.minw = minw;
    in.f0 = grid_h(sx, sy, tx, ty, minw, b->cfg.heuristic);
    in.est = 1000000ull + (uint64_t)w * h;
    b->insts.push_back(std::move(in));
    return (int)b->insts.size() - 1;
}

uint32_t gastar_batch_count(const gastar_batch* b) { return b ? (uint32_t)b->insts.size() : 0; }

}  // extern "C"

namespace {

int batch_upload(gastar_batch* b) {
    gastar_ctx* c = b->ctx;
    const uint32_t n = (uint32_t)b->insts.size();
    const auto& cf = b->cfg;
    const uint32_t W = cf.warps_per_block, ew = cf.expansion_width;
    b->threads = W * 32;
    uint32_t kinds = 0;
    for (auto& in : b->insts) kinds |= kind_bit(in.kind);
    b->smem = stage_smem_bytes(kKindsAll, W, ew);
    const int nb = occupancy_blocks(c, kKindsAll, b->threads, b->smem);
    if (nb <= 0) return GASTAR_CUDA_ERROR;
    b->blocks = cf.blocks ? cf.blocks : (uint32_t)(nb * c->sms);
    b->blocks = std::max(1u, std::min(b->blocks, n));

    // Partition sizes.
    const float lf = std::min(0.95f, std::max(0.1f, cf.load_factor));
    b->h_desc.assign(n, InstDesc());
    std::vector<uint64_t> part_off(n), part_bytes(n);
    uint64_t arena_bytes = 0, weights_bytes = 0;
    b->path_words = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const BatchInst& in = b->insts[i];
        InstDesc& d = b->h_desc[i];
        std::memset(&d, 0, sizeof(d));
        d.kind = in.kind;
        d.heuristic = cf.heuristic;
        d.moves = cf.moves;
        d.n = in.n;
        d.start0 = in.start0;
        d.start1 = in.start1;
        d.goal0 = in.goal0;
        d.goal1 = in.goal1;
        d.W = in.W;
        d.H = in.H;
        d.minw = in.minw;
        d.f0 = in.f0 == kInf ? 0 : in.f0;
        d.heaps = W;
        d.ew = ew;
        d.max_probe = 4096;
        d.max_exp = cf.max_expansions;
        d.timeout_ns = (uint64_t)cf.timeout_ms * 1000000ull;
        uint64_t states, table_bytes, entries;
        const uint32_t eb = entry_bytes(in.kind);
        if (in.kind == KIND_GRID) {
            states = (uint64_t)in.W * in.H;
            d.table_words = states;
            d.table_limit = ~0ull;
            table_bytes = states * 8;
            entries = std::max<uint64_t>(1 << 16, states);
            b->path_words += std::max<uint64_t>(1024, 4ull * (in.W + in.H));
            weights_bytes = (weights_bytes + 15) & ~15ull;
            b->insts[i].weights_off = weights_bytes;
            weights_bytes += states;
        } else {
            states = cf.sliding_states ? cf.sliding_states
                                       : (in.n == 3 ? 181440ull : (1ull << 20));
            const uint64_t slots = next_pow2((uint64_t)((double)states / lf) + 1);
            const uint32_t sw = key_words(in.kind) == 1 ? 2 : 4;
            d.table_words = slots * sw;
            d.table_mask = slots - 1;
            d.table_limit = (uint64_t)((double)slots * lf);
            table_bytes = d.table_words * 8;
            entries = states;
            b->path_words += 512ull * key_words(in.kind);
        }
        const uint64_t per_heap = (entries + W - 1) / W;
        const uint64_t cap_nodes = std::max<uint64_t>(4, (per_heap * 2 + 31) / 32);
        d.heap_cap = (uint32_t)cap_nodes;
        const uint64_t heap_bytes = (uint64_t)W * (cap_nodes + 1) * 32 * eb;
        part_off[i] = arena_bytes;
        part_bytes[i] = table_bytes + (uint64_t)W * 8 + 256 + heap_bytes;
        arena_bytes += (part_bytes[i] + 255) & ~255ull;
    }
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    if (arena_bytes + weights_bytes + (64ull << 20) > free_b) {
        set_error("batch partitions exceed free device memory");
        return GASTAR_OUT_OF_MEMORY;
    }
    if (!b->arena.ensure(arena_bytes) || !b->weights.ensure(std::max<uint64_t>(weights_bytes, 16)) ||
        !b->descs.ensure(sizeof(InstDesc) * n) || !b->ctls.ensure(sizeof(InstCtl) * (n + 1)) ||
        !b->order.ensure(sizeof(uint32_t) * n) || !b->counters.ensure(64) ||
        !b->paths.ensure(b->path_words * 8))
        return GASTAR_OUT_OF_MEMORY;
    b->device_bytes = arena_bytes + weights_bytes + b->path_words * 8 +
                      (sizeof(InstDesc) + sizeof(InstCtl)) * (size_t)n;
    char* base = reinterpret_cast<char*>(b->arena.p);
    InstCtl* ctl_base = reinterpret_cast<InstCtl*>(b->ctls.p);
    for (uint32_t i = 0; i < n; ++i) {
        InstDesc& d = b->h_desc[i];
        char* p = base + part_off[i];
        d.table = reinterpret_cast<unsigned long long*>(p);
        p += d.table_words * 8;
        d.heap_hdr = reinterpret_cast<uint32_t*>(p);
        p += (uint64_t)W * 8;
        p = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(p) + 255) & ~uintptr_t(255));
        d.heap_nodes = p;
        d.ctl = ctl_base + i;
        if (b->insts[i].kind == KIND_GRID)
            d.weights = reinterpret_cast<const uint8_t*>(b->weights.p) + b->insts[i].weights_off;
    }
    for (uint32_t i = 0; i < n; ++i) {
        const InstDesc& d = b->h_desc[i];
        const char* end = reinterpret_cast<const char*>(d.heap_nodes) +
                          (uint64_t)W * (d.heap_cap + 1) * 32 * entry_bytes(d.kind);
        if (end > base + part_off[i] + part_bytes[i]) {
            set_error("internal: partition layout overflow");
            return GASTAR_BAD_INPUT;
        }
    }
    // Largest estimated work first; puzzles in the other parity class of the
    // standard move set are unreachable and are not scheduled at all.
    std::vector<uint32_t> order;
    for (uint32_t i = 0; i < n; ++i)
        if (!(b->insts[i].kind != KIND_GRID && b->insts[i].f0 == kInf)) order.push_back(i);
    std::stable_sort(order.begin(), order.end(),
                     [&](uint32_t a, uint32_t bb) { return b->insts[a].est > b->insts[bb].est; });
    b->n_sched = (uint32_t)order.size();
    if (!b->h_ctl && !cuda_ok(cudaMallocHost(&b->h_ctl, sizeof(InstCtl) * (n + 1)), "cudaMallocHost"))
        return GASTAR_CUDA_ERROR;
    cudaStream_t st = c->stream;
    b->h2d = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const BatchInst& in = b->insts[i];
        if (in.kind != KIND_GRID) continue;
        if (!cuda_ok(cudaMemcpyAsync(reinterpret_cast<char*>(b->weights.p) + in.weights_off,
                                     in.weights.data(), in.weights.size(), cudaMemcpyHostToDevice, st),
                     "cudaMemcpyAsync"))
            return GASTAR_CUDA_ERROR;
        b->h2d += in.weights.size();
    }
    if (!cuda_ok(cudaMemcpyAsync(b->descs.p, b->h_desc.data(), sizeof(InstDesc) * n,
                                 cudaMemcpyHostToDevice, st), "cudaMemcpyAsync") ||
        (b->n_sched && !cuda_ok(cudaMemcpyAsync(b->order.p, order.data(), sizeof(uint32_t) * b->n_sched,
                                                cudaMemcpyHostToDevice, st), "cudaMemcpyAsync")) ||
        !cuda_ok(cudaStreamSynchronize(st), "cudaStreamSynchronize"))
        return GASTAR_CUDA_ERROR;
    b->h2d += sizeof(InstDesc) * n + sizeof(uint32_t) * n;
    b->uploaded = true;
    return GASTAR_OK;
}

// Enqueues one full solve of every instance on `st`.
int batch_enqueue(gastar_batch* b, cudaStream_t st, bool timed) {
    const uint32_t n = (uint32_t)b->insts.size();
    unsigned long long* used = reinterpret_cast<unsigned long long*>(b->counters.p) + 1;
    if (!cuda_ok(cudaMemsetAsync(b->ctls.p, 0, sizeof(InstCtl) * (n + 1), st), "cudaMemsetAsync") ||
        !cuda_ok(cudaMemsetAsync(b->counters.p, 0, 64, st), "cudaMemsetAsync"))
        return GASTAR_CUDA_ERROR;
    LaunchParams P;
    std::memset(&P, 0, sizeof(P));
    P.insts = reinterpret_cast<const InstDesc*>(b->descs.p);
    P.n_insts = b->n_sched;
    P.order = reinterpret_cast<const uint32_t*>(b->order.p);
    P.next = reinterpret_cast<uint32_t*>(b->counters.p);
    P.team_ctas = 1;
    P.barrier_timeout_ns = 2000000000ull;
    // External records stay timing events when the sequence is captured in a graph.
    if (timed && !cuda_ok(cudaEventRecordWithFlags(b->e0, st, cudaEventRecordExternal), "cudaEventRecord"))
        return GASTAR_CUDA_ERROR;
    int rc = launch_search(b->ctx, kKindsAll, P, b->blocks, b->threads, b->smem, st);
    if (rc != GASTAR_OK) return rc;
    if (timed && !cuda_ok(cudaEventRecordWithFlags(b->e1, st, cudaEventRecordExternal), "cudaEventRecord"))
        return GASTAR_CUDA_ERROR;
    rc = launch_paths(P.insts, n, reinterpret_cast<unsigned long long*>(b->paths.p), b->path_words, used, st);
    if (rc != GASTAR_OK) return rc;
    // Control blocks and the arena fill counter come back in one copy.
    if (!cuda_ok(cudaMemcpyAsync(reinterpret_cast<InstCtl*>(b->ctls.p) + n, b->counters.p, 16,
                                 cudaMemcpyDeviceToDevice, st), "cudaMemcpyAsync") ||
        !cuda_ok(cudaMemcpyAsync(b->h_ctl, b->ctls.p, sizeof(InstCtl) * (n + 1), cudaMemcpyDeviceToHost, st),
                 "cudaMemcpyAsync"))
        return GASTAR_CUDA_ERROR;
    return GASTAR_OK;
}

int batch_finish(gastar_batch* b) {
    cudaStream_t st = b->ctx->stream;
    if (!cuda_ok(cudaStreamSynchronize(st), "cudaStreamSynchronize")) return GASTAR_CUDA_ERROR;
    const uint32_t n = (uint32_t)b->insts.size();
    if (!cuda_ok(cudaEventElapsedTime(&b->kernel_ms, b->e0, b->e1), "cudaEventElapsedTime"))
        return GASTAR_CUDA_ERROR;
    b->d2h = sizeof(InstCtl) * (n + 1);
    // The arena counter (second word of the counters block) sits at h_ctl[n].
    const unsigned long long used = reinterpret_cast<const unsigned long long*>(&b->h_ctl[n])[1];
    const uint64_t words = std::min<uint64_t>(used, b->path_words);
    b->h_paths.resize(words);
    if (words) {
        if (!cuda_ok(cudaMemcpyAsync(b->h_paths.data(), b->paths.p, words * 8, cudaMemcpyDeviceToHost, st),
                     "cudaMemcpyAsync") ||
            !cuda_ok(cudaStreamSynchronize(st), "cudaStreamSynchronize"))
            return GASTAR_CUDA_ERROR;
        b->d2h += words * 8;
    }
    // Instances the standard move set cannot solve never ran a search.
    for (uint32_t i = 0; i < n; ++i)
        if (b->insts[i].kind != KIND_GRID && b->insts[i].f0 == kInf) {
            b->h_ctl[i].status = ST_NO_PATH;
            b->h_ctl[i].life = LIFE_DONE;
        }
    return GASTAR_OK;
}

}  // namespace

extern "C" {

int gastar_batch_run(gastar_batch* b) {
    if (!b) return GASTAR_BAD_INPUT;
    if (b->insts.empty()) return GASTAR_OK;
    if (cudaSetDevice(b->ctx->device) != cudaSuccess) return GASTAR_CUDA_ERROR;
    if (!b->uploaded) {
        int rc = batch_upload(b);
        if (rc != GASTAR_OK) return rc;
    }
    return gastar_batch_rerun(b);
}

int gastar_batch_rerun(gastar_batch* b) {
    if (!b || !b->uploaded) return GASTAR_BAD_INPUT;
    if (cudaSetDevice(b->ctx->device) != cudaSuccess) return GASTAR_CUDA_ERROR;
    cudaStream_t st = b->ctx->stream;
    if (b->cfg.use_graph) {
        if (!b->graph) {
            cudaGraph_t g;
            if (!cuda_ok(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture"))
                return GASTAR_CUDA_ERROR;
            int rc = batch_enqueue(b, st, true);
            cudaError_t ce = cudaStreamEndCapture(st, &g);
            if (rc != GASTAR_OK) return rc;
            if (!cuda_ok(ce, "cudaStreamEndCapture")) return GASTAR_CUDA_ERROR;
            ce = cudaGraphInstantiate(&b->graph, g, 0);
            cudaGraphDestroy(g);
            if (!cuda_ok(ce, "cudaGraphInstantiate")) return GASTAR_CUDA_ERROR;
        }
        if (!cuda_ok(cudaGraphLaunch(b->graph, st), "cudaGraphLaunch")) return GASTAR_CUDA_ERROR;
    } else {
        int rc = batch_enqueue(b, st, true);
        if (rc != GASTAR_OK) return rc;
    }
    return batch_finish(b);
}

int gastar_batch_result(gastar_batch* b, uint32_t i, gastar_result* out) {
    if (!b || !out || i >= b->insts.size() || !b->h_ctl) return GASTAR_BAD_INPUT;
    std::memset(out, 0, sizeof(*out));
    const InstCtl& c = b->h_ctl[i];
    out->status = (int32_t)c.status;
    out->cost = c.status == ST_OK ? c.best : 0;
    out->path_len = c.path_len;
    out->iterations = c.iterations;
    out->expansions = c.expansions;
    out->generated = c.generated;
    out->pushes = c.pushes;
    out->stale = c.stale;
    out->table_used = c.table_used;
    out->kernel_ms = b->kernel_ms;
    out->attempts = 1;
    return GASTAR_OK;
}

int gastar_batch_path(gastar_batch* b, uint32_t i, void* path, uint32_t cap, uint32_t* len) {
    if (!b || i >= b->insts.size() || !b->h_ctl) return GASTAR_BAD_INPUT;
    const InstCtl& c = b->h_ctl[i];
    if (len) *len = c.status == ST_OK ? c.path_len : 0;
    if (c.status != ST_OK) return GASTAR_OK;
    if (c.path_len > cap) return GASTAR_PATH_CAP;
    const BatchInst& in = b->insts[i];
    const uint32_t kw = key_words(in.kind);
    if (c.path_off + (uint64_t)c.path_len * kw > b->h_paths.size()) return GASTAR_PATH_CAP;
    const unsigned long long* src = b->h_paths.data() + c.path_off;
    for (uint32_t s = 0; s < c.path_len; ++s) {
        const uint32_t j = c.path_len - 1 - s;  // stored goal-first
        if (in.kind == KIND_GRID) {
            reinterpret_cast<uint32_t*>(path)[s] = (uint32_t)src[j];
        } else {
            unpack_board(in.n, src[(size_t)j * kw], kw == 2 ? src[(size_t)j * kw + 1] : 0,
                         reinterpret_cast<uint8_t*>(path) + (size_t)s * in.n * in.n);
        }
    }
    return GASTAR_OK;
}

int gastar_batch_stats(gastar_batch* b, float* kernel_ms, uint64_t* h2d, uint64_t* d2h, uint64_t* dev) {
    if (!b) return GASTAR_BAD_INPUT;
    if (kernel_ms) *kernel_ms = b->kernel_ms;
    if (h2d) *h2d = b->h2d;
    if (d2h) *d2h = b->d2h;
    if (dev) *dev = b->device_bytes;
    return GASTAR_OK;
}

}  // extern "C"
