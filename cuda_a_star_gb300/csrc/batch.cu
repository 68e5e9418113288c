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
#include <cmath>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/gastar.h"
#include "device_common.cuh"
#include "engine_internal.h"
#include "partition.h"

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

// Copies a grid from host memory that the GPU reads in place (pageable
// memory through the host's page tables) and reduces its least passable
// weight in the same pass: per byte, min(w - 1) with 0 (obstacle) wrapping to
// 0xff, 16 bytes per load where both pointers allow it.
__global__ void copy_min_kernel(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, uint64_t cells,
                                uint32_t* out) {
    uint32_t m = 0xffffffffu;
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t nth = (uint64_t)gridDim.x * blockDim.x;
    uint64_t done = 0;
    if ((((uintptr_t)src | (uintptr_t)dst) & 15) == 0) {
        const uint64_t n16 = cells / 16;
        const uint4* s = reinterpret_cast<const uint4*>(src);
        uint4* d = reinterpret_cast<uint4*>(dst);
        for (uint64_t i = tid; i < n16; i += nth) {
            const uint4 v = s[i];
            d[i] = v;
            m = __vminu4(m, __vsub4(v.x, 0x01010101u));
            m = __vminu4(m, __vsub4(v.y, 0x01010101u));
            m = __vminu4(m, __vsub4(v.z, 0x01010101u));
            m = __vminu4(m, __vsub4(v.w, 0x01010101u));
        }
        done = n16 * 16;
    }
    for (uint64_t i = done + tid; i < cells; i += nth) {
        const uint32_t b = src[i];
        dst[i] = (uint8_t)b;
        m = __vminu4(m, ((b - 1u) & 0xffu) | 0xffffff00u);
    }
    uint32_t r = min(min(m & 0xffu, (m >> 8) & 0xffu), min((m >> 16) & 0xffu, m >> 24));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r = min(r, __shfl_xor_sync(kFull, r, o));
    if ((threadIdx.x & 31) == 0 && r != 0xffu) atomicMin(out, r);
}

int upload_grid(gastar_ctx* c, uint8_t* d_dst, const uint8_t* h_src, uint64_t cells, cudaStream_t st,
                uint32_t* minw) {
    if (c->upload_mode == 2) {
        const int rc = upload_grid_staged(c, d_dst, h_src, cells, st, minw);
        if (rc != GASTAR_OUT_OF_MEMORY) return rc;  // no pinned ring: copy
    }
    if (c->upload_mode != 1) {
        if (!cuda_ok(cudaMemcpyAsync(d_dst, h_src, cells, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync"))
            return GASTAR_CUDA_ERROR;
        return device_min_weight(c, d_dst, cells, st, minw);
    }
    if (!c->misc.ensure(64)) return GASTAR_OUT_OF_MEMORY;
    uint32_t* d = reinterpret_cast<uint32_t*>(c->misc.p) + 9;
    const uint32_t init = 0xffu;
    if (!cuda_ok(cudaMemcpyAsync(d, &init, 4, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync"))
        return GASTAR_CUDA_ERROR;
    const uint64_t blocks = std::min<uint64_t>((cells / 16 + 255) / 256, (uint64_t)c->sms * 8);
    copy_min_kernel<<<(unsigned)std::max<uint64_t>(1, blocks), 256, 0, st>>>(h_src, d_dst, cells, d);
    if (!cuda_ok(cudaGetLastError(), "copy_min_kernel")) return GASTAR_CUDA_ERROR;
    uint32_t r = 0xffu;
    if (!cuda_ok(cudaMemcpyAsync(&r, d, 4, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync") ||
        !cuda_ok(cudaStreamSynchronize(st), "cudaStreamSynchronize"))
        return GASTAR_CUDA_ERROR;
    *minw = r == 0xffu ? 255u : r + 1u;
    return GASTAR_OK;
}

}  // namespace gastar

using namespace gastar;

struct gastar_batch;
namespace gastar {
uint8_t* grid_alloc(gastar_batch* b, size_t bytes);
}

struct gastar_batch {
    gastar_ctx* ctx = nullptr;
    gastar_batch_config cfg;
    std::vector<Problem> insts;
    // Grid weights, copied to the device when the grid is added: bump
    // allocation in chunks of at least 256 MiB, freed with the batch.
    // Re-run batches and autotuner trials point at their parent's copies.
    std::vector<void*> grid_chunks;
    size_t grid_chunk_used = 0, grid_chunk_cap = 0;
    uint64_t grid_bytes = 0, grid_h2d = 0;
    std::vector<uint8_t> heavy;        // solved by a multi-block team
    std::vector<uint8_t> promotable;   // re-solved by the plain engine past the budget
    uint32_t n_heavy = 0, heavy_teams = 0;
    uint64_t heavy_stage_bytes = 0;
    uint32_t heap_snodes = kHeapSmemNodes;  // shared-memory heap nodes per warp
    DevBuf team_ctl, team_stage;
    uint32_t promoted = 0;
    float main_ms = 0, retry_ms = 0, promote_ms = 0;  // kernel time by phase of the last run
    uint32_t retry_level = 0;   // partitions scale by 4^retry_level
    uint32_t retried = 0;       // instances re-solved with larger partitions in the last run
    double block_share = 0;     // > 0: use this share of the resident blocks (autotuner trials)
    gastar_batch* sub = nullptr;    // re-run batch of the last run's overflowed instances,
    std::vector<uint32_t> sub_idx;  // kept while the same instances overflow
    bool uploaded = false;
    DevBuf arena, descs, ctls, order, counters, paths;
    DevBuf tcounts;  // per instance: length of its partition's claim list
    std::vector<InstDesc> h_desc;
    std::vector<uint64_t> tl_start, tl_end;  // the persistent launch's schedule (globaltimer ns)
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

namespace gastar {

uint8_t* grid_alloc(gastar_batch* b, size_t bytes) {
    bytes = (bytes + 255) & ~(size_t)255;
    if (b->grid_chunks.empty() || b->grid_chunk_used + bytes > b->grid_chunk_cap) {
        const size_t cap = std::max<size_t>(bytes, (size_t)256 << 20);
        void* c = nullptr;
        if (cudaMalloc(&c, cap) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        b->grid_chunks.push_back(c);
        b->grid_chunk_cap = cap;
        b->grid_chunk_used = 0;
        b->grid_bytes += cap;
    }
    uint8_t* r = static_cast<uint8_t*>(b->grid_chunks.back()) + b->grid_chunk_used;
    b->grid_chunk_used += bytes;
    return r;
}

}  // namespace gastar

extern "C" {

void gastar_batch_config_default(gastar_batch_config* cfg) {
    std::memset(cfg, 0, sizeof(*cfg));
    // The autotuner's usual choice on mixed puzzle/grid batches.
    cfg->warps_per_block = 16;
    cfg->expansion_width = 32;
    cfg->load_factor = 0.5f;
    cfg->heuristic = GASTAR_H_ADMISSIBLE;
    cfg->moves = GASTAR_MOVES_STANDARD;
    cfg->use_graph = 1;
    cfg->delta_grid = 9;
    cfg->heavy_team = 2;
    cfg->heavy_cells = 1ull << 21;
    cfg->promote_expansions = 1ull << 21;
    cfg->open_list = 1;
}

gastar_batch* gastar_batch_create(gastar_ctx* c, const gastar_batch_config* cfg) {
    if (!c) return nullptr;
    auto* b = new gastar_batch();
    b->ctx = c;
    if (cfg) b->cfg = *cfg;
    else gastar_batch_config_default(&b->cfg);
    if (!b->cfg.heavy_team) b->cfg.heavy_team = 1;
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
    gastar_batch_destroy(b->sub);
    b->arena.release();
    for (void* c : b->grid_chunks) cudaFree(c);
    b->descs.release();
    b->ctls.release();
    b->order.release();
    b->counters.release();
    b->paths.release();
    b->tcounts.release();
    b->team_ctl.release();
    b->team_stage.release();
    if (b->h_ctl) cudaFreeHost(b->h_ctl);
    if (b->e0) cudaEventDestroy(b->e0);
    if (b->e1) cudaEventDestroy(b->e1);
    delete b;
}

int gastar_batch_add_sliding(gastar_batch* b, uint32_t n, const uint8_t* start, const uint8_t* goal) {
    if (!b || b->uploaded) return -GASTAR_BAD_INPUT;
    Problem p;
    if (!make_sliding_problem(n, start, goal, b->cfg.heuristic, b->cfg.moves, p)) {
        set_error("sliding: boards must be permutations of 0..n*n-1 with n in 3..5");
        return -GASTAR_BAD_INPUT;
    }
    b->insts.push_back(std::move(p));
    return (int)b->insts.size() - 1;
}

// The grid goes straight from the caller's buffer to the device (no host
// copy: first-touch page faults of a host copy cost more than the transfer),
// and its least passable weight is reduced there.
int gastar_batch_add_grid(gastar_batch* b, uint32_t w, uint32_t h, const uint8_t* weights, uint32_t sx,
                          uint32_t sy, uint32_t tx, uint32_t ty) {
    if (!b || b->uploaded) return -GASTAR_BAD_INPUT;
    Problem p;
    if (!make_grid_problem(w, h, weights, sx, sy, tx, ty, b->cfg.heuristic, p, false)) {
        set_error("grid: bad dimensions or endpoints");
        return -GASTAR_BAD_INPUT;
    }
    if (cudaSetDevice(b->ctx->device) != cudaSuccess) return -GASTAR_CUDA_ERROR;
    const size_t cells = (size_t)w * h;
    uint8_t* d = grid_alloc(b, cells);
    if (!d) {
        set_error("batch: grid weights exceed free device memory");
        return -GASTAR_OUT_OF_MEMORY;
    }
    cudaStream_t st = b->ctx->stream;
    uint32_t mw = 255;
    const int rc = upload_grid(b->ctx, d, weights, cells, st, &mw);
    if (rc != GASTAR_OK) return -rc;
    set_grid_minw(p, mw, b->cfg.heuristic);
    p.d_weights = d;
    b->grid_h2d += cells;
    b->insts.push_back(std::move(p));
    return (int)b->insts.size() - 1;
}

uint32_t gastar_batch_count(const gastar_batch* b) { return b ? (uint32_t)b->insts.size() : 0; }

}  // extern "C"

namespace {

PartConfig part_config(const gastar_batch* b) {
    PartConfig pc;
    const auto& cf = b->cfg;
    pc.warps = cf.warps_per_block;
    pc.ew = cf.expansion_width;
    pc.load_factor = cf.load_factor;
    pc.heuristic = cf.heuristic;
    pc.moves = cf.moves;
    pc.delta_grid = cf.delta_grid;
    pc.sliding_states = cf.sliding_states;
    pc.max_exp = cf.max_expansions;
    pc.timeout_ms = cf.timeout_ms;
    pc.retry_level = b->retry_level;
    pc.heap_snodes = b->heap_snodes;
    pc.buckets = cf.open_list == 1;
    pc.claim_list = true;  // re-runs clear only the slots the last search claimed
    return pc;
}

int batch_upload(gastar_batch* b) {
    gastar_ctx* c = b->ctx;
    const uint32_t n = (uint32_t)b->insts.size();
    PartConfig pc = part_config(b);
    b->threads = pc.warps * 32;
    // Shared memory for the kinds in the batch (one kernel serves all kinds).
    uint32_t present = 0;
    for (const Problem& p : b->insts) present |= kind_bit(p.kind);
    b->smem = block_smem_bytes(present, pc.warps, pc.ew, false, kHeapSmemNodes, pc.buckets);
    if (b->smem + 4096 > c->smem_optin) {  // + the kernel's static shared memory
        set_error("batch: warps_per_block x expansion_width needs more shared memory than a block has");
        return GASTAR_OUT_OF_MEMORY;
    }
    const int nb = occupancy_blocks(c, kKindsAll, b->threads, b->smem);
    if (nb <= 0) return GASTAR_CUDA_ERROR;
    // The heaps' top levels take the shared memory the resident blocks leave.
    b->heap_snodes = fit_heap_snodes(c, present, pc.warps, pc.ew, false, b->threads, nb, &b->smem, pc.buckets);
    pc.heap_snodes = b->heap_snodes;
    b->blocks = b->cfg.blocks ? b->cfg.blocks : (uint32_t)(nb * c->sms);
    if (b->block_share > 0)
        b->blocks = std::max(1u, (uint32_t)((double)nb * c->sms * b->block_share + 0.5));
    b->blocks = std::max(1u, std::min(b->blocks, n));

    // Heavy instances (large grids) are solved by teams of heavy_team blocks;
    // their partitions hold heavy_team x warps warp-heaps.
    const uint32_t T = std::max(1u, b->cfg.heavy_team);
    PartConfig pch = pc;
    pch.warps = pc.warps * T;
    b->heavy.assign(n, 0);
    b->promotable.assign(n, 0);
    b->n_heavy = 0;
    uint64_t heavy_est = 0, total_est = 0, heavy_min = ~0ull;
    for (uint32_t i = 0; i < n; ++i) {
        const Problem& p = b->insts[i];
        const uint64_t work = p.est;
        total_est += work;
        if (T > 1 && p.kind == KIND_GRID && (uint64_t)p.W * p.H >= b->cfg.heavy_cells) {
            b->heavy[i] = 1;
            ++b->n_heavy;
            heavy_est += work;
            heavy_min = std::min(heavy_min, work);
        }
        const uint64_t pe = b->cfg.promote_expansions;
        if (p.kind != KIND_GRID && p.n >= 4 && pe && (!b->cfg.max_expansions || b->cfg.max_expansions > pe))
            b->promotable[i] = 1;
    }
    b->heavy_teams = 0;
    if (b->n_heavy) {
        // Enough teams that the heavy queue, whose instances each hold a team
        // for est / T, ends no later than the one-block queue: the heavy work
        // over the expected makespan less the time of the last (smallest)
        // heavy instance, which a team takes when the others are nearly done.
        // Teams that run out of heavy instances take one-block instances, so a
        // team too many costs little; a team too few leaves the heavy
        // instances as the tail.
        const double M = (double)total_est / b->blocks;
        const double tail = (double)heavy_min / T;
        const double need = (double)heavy_est / std::max(M - tail, 0.5 * M);
        b->heavy_teams = (uint32_t)std::max<double>(1.0, std::ceil(need / T));
        b->heavy_teams = std::min(b->heavy_teams, b->n_heavy);
        b->heavy_teams = std::min(b->heavy_teams, b->blocks / T);
        if (b->heavy_teams == 0) {  // too few blocks for a team: no teams
            b->n_heavy = 0;
            std::fill(b->heavy.begin(), b->heavy.end(), 0);
        }
    }
    std::vector<PartPlan> plans(n);
    std::vector<uint64_t> part_off(n);
    uint64_t arena_bytes = 0;
    b->path_words = 0;
    for (uint32_t i = 0; i < n; ++i) {
        plans[i] = plan_partition(b->insts[i], b->heavy[i] ? pch : pc);
        part_off[i] = arena_bytes;
        arena_bytes += plans[i].bytes;
        b->path_words += plans[i].path_words;
    }
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    if (arena_bytes + (64ull << 20) > free_b) {
        set_error("batch partitions exceed free device memory");
        return GASTAR_OUT_OF_MEMORY;
    }
    if (!b->arena.ensure(arena_bytes) || !b->descs.ensure(sizeof(InstDesc) * n) || !b->ctls.ensure(sizeof(InstCtl) * (n + 1)) ||
        !b->order.ensure(sizeof(uint32_t) * n) || !b->counters.ensure(64) ||
        !b->paths.ensure(b->path_words * 8) || !b->tcounts.ensure(sizeof(unsigned long long) * n))
        return GASTAR_OUT_OF_MEMORY;
    b->device_bytes = arena_bytes + b->grid_bytes + b->path_words * 8 +
                      (sizeof(InstDesc) + sizeof(InstCtl)) * (size_t)n;
    char* base = reinterpret_cast<char*>(b->arena.p);
    InstCtl* ctl_base = reinterpret_cast<InstCtl*>(b->ctls.p);
    unsigned long long* tcount = reinterpret_cast<unsigned long long*>(b->tcounts.p);
    b->h_desc.assign(n, InstDesc());
    for (uint32_t i = 0; i < n; ++i) {
        fill_desc(b->h_desc[i], b->insts[i], b->heavy[i] ? pch : pc, plans[i], base + part_off[i],
                  b->insts[i].d_weights, ctl_base + i, tcount + i);
        if (b->promotable[i])
            b->h_desc[i].max_exp = b->h_desc[i].max_exp ? std::min<uint64_t>(b->h_desc[i].max_exp,
                                                                              b->cfg.promote_expansions)
                                                        : b->cfg.promote_expansions;
    }
    // Largest estimated work first; puzzles in the other parity class of the
    // standard move set are unreachable and are not scheduled at all.  The
    // order array holds the one-block instances, then the heavy ones.
    std::vector<uint32_t> order, horder;
    for (uint32_t i = 0; i < n; ++i) {
        if (b->insts[i].unreachable) continue;
        (b->heavy[i] ? horder : order).push_back(i);
    }
    auto by_est = [&](uint32_t a, uint32_t bb) { return sched_before(b->insts[a], b->insts[bb]); };
    std::stable_sort(order.begin(), order.end(), by_est);
    std::stable_sort(horder.begin(), horder.end(), by_est);
    b->n_sched = (uint32_t)order.size();
    order.insert(order.end(), horder.begin(), horder.end());
    if (b->n_heavy) {
        b->heavy_stage_bytes = team_stage_bytes(T, pc.warps, pc.ew, 8, 16);
        if (!b->team_ctl.ensure(sizeof(TeamCtl) * b->heavy_teams) ||
            !b->team_stage.ensure(b->heavy_stage_bytes * b->heavy_teams))
            return GASTAR_OUT_OF_MEMORY;
    }
    if (!b->h_ctl && !cuda_ok(cudaMallocHost(&b->h_ctl, sizeof(InstCtl) * (n + 1)), "cudaMallocHost"))
        return GASTAR_CUDA_ERROR;
    cudaStream_t st = c->stream;
    b->h2d = b->grid_h2d;  // the grids went up when they were added
    // The partitions' contents are unknown: every claim-list length starts
    // above its capacity, so each table's first search clears it whole.
    if (!cuda_ok(cudaMemsetAsync(b->tcounts.p, 0xff, sizeof(unsigned long long) * n, st), "cudaMemsetAsync"))
        return GASTAR_CUDA_ERROR;
    if (!cuda_ok(cudaMemcpyAsync(b->descs.p, b->h_desc.data(), sizeof(InstDesc) * n,
                                 cudaMemcpyHostToDevice, st), "cudaMemcpyAsync") ||
        (!order.empty() && !cuda_ok(cudaMemcpyAsync(b->order.p, order.data(), sizeof(uint32_t) * order.size(),
                                                    cudaMemcpyHostToDevice, st), "cudaMemcpyAsync")) ||
        !cuda_ok(cudaStreamSynchronize(st), "cudaStreamSynchronize"))
        return GASTAR_CUDA_ERROR;
    b->h2d += sizeof(InstDesc) * n + sizeof(uint32_t) * n;
    b->uploaded = true;
    return GASTAR_OK;
}

// Enqueues one full solve of every instance on `st`.
int batch_enqueue(gastar_batch* b, cudaStream_t st, bool capturing) {
    const uint32_t n = (uint32_t)b->insts.size();
    unsigned long long* used = reinterpret_cast<unsigned long long*>(b->counters.p) + 1;
    if (!cuda_ok(cudaMemsetAsync(b->ctls.p, 0, sizeof(InstCtl) * (n + 1), st), "cudaMemsetAsync") ||
        !cuda_ok(cudaMemsetAsync(b->counters.p, 0, 64, st), "cudaMemsetAsync"))
        return GASTAR_CUDA_ERROR;
    LaunchParams P;
    std::memset(&P, 0, sizeof(P));
    P.insts = reinterpret_cast<const InstDesc*>(b->descs.p);
    P.n_insts = b->n_sched;
    P.heap_snodes = b->heap_snodes;
    P.buckets = b->cfg.open_list == 1 ? 1u : 0u;
    P.order = reinterpret_cast<const uint32_t*>(b->order.p);
    P.next = reinterpret_cast<uint32_t*>(b->counters.p);
    P.team_ctas = 1;
    P.barrier_timeout_ns = 2000000000ull;
    if (b->n_heavy) {
        P.heavy_order = reinterpret_cast<const uint32_t*>(b->order.p) + b->n_sched;
        P.n_heavy = b->n_heavy;
        P.heavy_team = b->cfg.heavy_team;
        P.heavy_teams = b->heavy_teams;
        P.heavy_next = reinterpret_cast<uint32_t*>(b->counters.p) + 4;
        P.heavy_ctl = reinterpret_cast<TeamCtl*>(b->team_ctl.p);
        P.heavy_stage = b->team_stage.p;
        P.heavy_stage_bytes = b->heavy_stage_bytes;
        if (!cuda_ok(cudaMemsetAsync(b->team_ctl.p, 0, sizeof(TeamCtl) * b->heavy_teams, st), "cudaMemsetAsync"))
            return GASTAR_CUDA_ERROR;
    }
    // Inside a graph capture, external records stay timing events.
    const unsigned flags = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    if (!cuda_ok(cudaEventRecordWithFlags(b->e0, st, flags), "cudaEventRecord")) return GASTAR_CUDA_ERROR;
    int rc = launch_search(b->ctx, kKindsAll, P, b->blocks, b->threads, b->smem, st);
    if (rc != GASTAR_OK) return rc;
    if (!cuda_ok(cudaEventRecordWithFlags(b->e1, st, flags), "cudaEventRecord")) return GASTAR_CUDA_ERROR;
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
    b->retry_ms = b->promote_ms = 0;
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
    b->tl_start.resize(n);
    b->tl_end.resize(n);
    for (uint32_t i = 0; i < n; ++i) {
        b->tl_start[i] = b->h_ctl[i].t_start;
        b->tl_end[i] = b->h_ctl[i].t_end;
    }
    // Instances the standard move set cannot solve never ran a search.
    for (uint32_t i = 0; i < n; ++i)
        if (b->insts[i].unreachable) {
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

namespace {

// Re-solves the instances whose partition overflowed (or whose path did not
// fit the arena) in a follow-up batch with 4x larger partitions, then merges
// their control blocks and paths back.  The follow-up batch retries its own
// overflows the same way, down to 64x the class size, and is kept for the
// next run while the same instances overflow (a rerun replays it without new
// allocations or uploads).
// Few overflowed instances are left to the plain engine (re-solved one at a
// time on the whole GPU with a growing table, see batch_promote): a second
// batch launch over a handful of instances would keep most SMs idle.
constexpr uint32_t kPlainOverflowMax = 64;

bool overflowed(uint32_t st) { return st == ST_TABLE_FULL || st == ST_HEAP_FULL || st == ST_PATH_CAP; }

int batch_retry_overflows(gastar_batch* b) {
    b->retried = 0;
    if (b->retry_level >= 3) return GASTAR_OK;
    const uint32_t n = (uint32_t)b->insts.size();
    std::vector<uint32_t> bad;
    for (uint32_t i = 0; i < n; ++i)
        if (overflowed(b->h_ctl[i].status)) bad.push_back(i);
    if (bad.size() <= kPlainOverflowMax) return GASTAR_OK;
    const bool fresh = !b->sub || b->sub_idx != bad;
    if (fresh) {
        gastar_batch_destroy(b->sub);
        b->sub = gastar_batch_create(b->ctx, &b->cfg);
        b->sub_idx.clear();
        if (!b->sub) return GASTAR_OUT_OF_MEMORY;
        b->sub->cfg.use_graph = 0;
        b->sub->retry_level = b->retry_level + 1;
        for (uint32_t i : bad) b->sub->insts.push_back(b->insts[i]);
        b->sub_idx = bad;
    }
    gastar_batch* sub = b->sub;
    int rc = gastar_batch_run(sub);
    if (rc == GASTAR_OK) {
        b->retried = (uint32_t)bad.size();
        for (size_t j = 0; j < bad.size(); ++j) {
            InstCtl c = sub->h_ctl[j];
            c.iterations += b->h_ctl[bad[j]].iterations;
            c.expansions += b->h_ctl[bad[j]].expansions;
            if (c.status == ST_OK) {
                const uint64_t words = (uint64_t)c.path_len * key_words(b->insts[bad[j]].kind);
                const uint64_t off = b->h_paths.size();
                b->h_paths.insert(b->h_paths.end(), sub->h_paths.begin() + c.path_off,
                                  sub->h_paths.begin() + c.path_off + words);
                c.path_off = off;
            }
            b->h_ctl[bad[j]] = c;
        }
        b->kernel_ms += sub->kernel_ms;
        b->retry_ms += sub->kernel_ms;
        if (fresh) b->h2d += sub->h2d;  // a kept re-run batch uploads nothing again
        b->d2h += sub->d2h;
    } else {
        gastar_batch_destroy(b->sub);
        b->sub = nullptr;
        b->sub_idx.clear();
    }
    return rc;
}

}  // namespace

// Puzzles that used up their promotion budget in the batch, and instances
// that overflowed their partitions (when there are few of them), are solved
// again from scratch by the plain engine: one instance on every block of the
// GPU, its table growing as needed.
static int batch_promote(gastar_batch* b) {
    b->promoted = 0;
    const uint32_t n = (uint32_t)b->insts.size();
    for (uint32_t i = 0; i < n; ++i) {
        const bool budget = b->promotable[i] && b->h_ctl[i].status == ST_BUDGET;
        if (!budget && !overflowed(b->h_ctl[i].status)) continue;
        const Problem& p = b->insts[i];
        PlainProblem pp;
        std::memset(&pp, 0, sizeof(pp));
        pp.kind = p.kind;
        pp.n = p.n;
        pp.start0 = p.start0;
        pp.start1 = p.start1;
        pp.goal0 = p.goal0;
        pp.goal1 = p.goal1;
        pp.f0 = p.f0;
        if (p.kind == KIND_GRID) {  // the grid's weights are already on the device
            pp.W = p.W;
            pp.H = p.H;
            pp.minw = p.minw;
            pp.d_weights = p.d_weights;
        }
        gastar_config cfg;
        gastar_config_default(&cfg);
        // Puzzles re-solved here passed their budget: a few million
        // expansions, so an iteration's pops, not the depth, set the
        // iteration count.  65536 parallel pops: the batched mix's 36 hardest
        // 15-puzzles in 87 iterations each and 75 ms in all, against 155
        // iterations and 106 ms at 16384.
        cfg.num_queues = p.kind == KIND_GRID ? 16384 : 65536;
        cfg.heuristic = b->cfg.heuristic;
        cfg.moves = b->cfg.moves;
        cfg.timeout_ms = b->cfg.timeout_ms;
        if (b->cfg.max_expansions) cfg.max_expansions = b->cfg.max_expansions;
        if (p.kind == KIND_GRID) {
            cfg.delta = b->cfg.delta_grid;
        } else {
            // It outgrew its partition or its budget: start large, one attempt.
            cfg.table_log2 = p.kind == KIND_SLIDING5 ? 27 : 26;
            cfg.heap_entries = 1ull << 25;
        }
        std::vector<uint64_t> keys;
        gastar_result r;
        std::memset(&r, 0, sizeof(r));
        const int rc = plain_solve(b->ctx, pp, &cfg, &keys, &r);
        if (rc != GASTAR_OK) return rc;
        InstCtl& c = b->h_ctl[i];
        const uint64_t batch_exp = c.expansions, t0 = c.t_start;
        c.status = (uint32_t)r.status;
        c.best = r.cost;
        c.path_len = r.status == GASTAR_OK ? r.path_len : 0;
        c.iterations += r.iterations;
        c.expansions = batch_exp + r.expansions;
        c.generated += r.generated;
        c.pushes += r.pushes;
        c.stale += r.stale;
        c.table_used = r.table_used;
        c.t_end = c.t_end + (uint64_t)((double)r.kernel_ms * 1e6);
        c.t_start = t0;
        if (r.status == GASTAR_OK) {
            c.path_off = b->h_paths.size();
            b->h_paths.insert(b->h_paths.end(), keys.begin(), keys.end());
        }
        b->kernel_ms += r.kernel_ms;
        b->promote_ms += r.kernel_ms;
        ++b->promoted;
    }
    return GASTAR_OK;
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
        int rc = batch_enqueue(b, st, false);
        if (rc != GASTAR_OK) return rc;
    }
    int rc = batch_finish(b);
    if (rc != GASTAR_OK) return rc;
    rc = batch_retry_overflows(b);
    if (rc != GASTAR_OK) return rc;
    return batch_promote(b);
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
    // Per-instance device time from its first iteration to its last.
    out->kernel_ms = c.t_end > c.t_start ? (float)((double)(c.t_end - c.t_start) * 1e-6) : 0.f;
    out->total_ms = b->kernel_ms;
    out->attempts = 1;
    out->launches = 2;
    return GASTAR_OK;
}

int gastar_batch_path(gastar_batch* b, uint32_t i, void* path, uint32_t cap, uint32_t* len) {
    if (!b || i >= b->insts.size() || !b->h_ctl) return GASTAR_BAD_INPUT;
    const InstCtl& c = b->h_ctl[i];
    if (len) *len = c.status == ST_OK ? c.path_len : 0;
    if (c.status != ST_OK) return GASTAR_OK;
    if (c.path_len > cap) return GASTAR_PATH_CAP;
    const Problem& in = b->insts[i];
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

int gastar_batch_phases(gastar_batch* b, float* main_ms, float* retry_ms, float* promote_ms, uint32_t* retried,
                        uint32_t* promoted) {
    if (!b) return GASTAR_BAD_INPUT;
    if (main_ms) *main_ms = b->kernel_ms - b->retry_ms - b->promote_ms;
    if (retry_ms) *retry_ms = b->retry_ms;
    if (promote_ms) *promote_ms = b->promote_ms;
    if (retried) *retried = b->retried;
    if (promoted) *promoted = b->promoted;
    return GASTAR_OK;
}

int gastar_batch_timeline(gastar_batch* b, uint64_t* start_ns, uint64_t* end_ns) {
    if (!b || !start_ns || !end_ns || b->tl_start.size() != b->insts.size()) return GASTAR_BAD_INPUT;
    const size_t n = b->tl_start.size();
    uint64_t t0 = ~0ull;
    for (size_t i = 0; i < n; ++i)
        if (b->tl_start[i] && b->tl_end[i] >= b->tl_start[i]) t0 = std::min(t0, b->tl_start[i]);
    for (size_t i = 0; i < n; ++i) {
        const bool ran = b->tl_start[i] && b->tl_end[i] >= b->tl_start[i];
        start_ns[i] = ran ? b->tl_start[i] - t0 : 0;
        end_ns[i] = ran ? b->tl_end[i] - t0 : 0;
    }
    return GASTAR_OK;
}

int gastar_batch_stats(gastar_batch* b, float* kernel_ms, uint64_t* h2d, uint64_t* d2h, uint64_t* dev) {
    if (!b) return GASTAR_BAD_INPUT;
    if (kernel_ms) *kernel_ms = b->kernel_ms;
    if (h2d) *h2d = b->h2d;
    if (d2h) *d2h = b->d2h;
    if (dev) {  // with the kept re-run batches
        *dev = 0;
        for (const gastar_batch* x = b; x; x = x->sub) *dev += x->device_bytes;
    }
    return GASTAR_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Autotuner: picks queue count (warp-heaps per instance), expansion width,
// table load factor, grid pop window and heavy-team size for the instance mix
// of a batch by timing trial batches over a stratified sample of its
// instances (coordinate descent from the current configuration).  Results are
// cached per GPU and mix signature in a text file.
// ---------------------------------------------------------------------------
namespace {

std::string mix_signature(const gastar_batch* b) {
    uint64_t counts[4] = {0, 0, 0, 0}, cells = 0, big = 0;
    for (const Problem& p : b->insts) {
        counts[p.kind] += 1;
        if (p.kind == KIND_GRID) {
            cells += (uint64_t)p.W * p.H;
            big += (uint64_t)p.W * p.H >= b->cfg.heavy_cells;
        }
    }
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s|sm%d|s3:%llu|s4:%llu|s5:%llu|g:%llu|cells:%llu|big:%llu|h%u|m%u",
                  b->ctx->name, b->ctx->sms, (unsigned long long)counts[0], (unsigned long long)counts[1],
                  (unsigned long long)counts[2], (unsigned long long)counts[3],
                  (unsigned long long)(counts[3] ? cells / counts[3] : 0), (unsigned long long)big,
                  b->cfg.heuristic, b->cfg.moves);
    for (char* c = buf; *c; ++c)
        if (*c == ' ' || *c == '\t') *c = '_';
    return buf;
}

bool cache_lookup(const char* path, const std::string& sig, gastar_batch_config& cfg) {
    if (!path) return false;
    FILE* f = std::fopen(path, "r");
    if (!f) return false;
    char line[1024];
    bool found = false;
    while (std::fgets(line, sizeof(line), f)) {
        char key[600];
        unsigned w, ew, dg, team;
        float lf;
        unsigned ol = 0;
        unsigned long long hc = 0;
        const int got = std::sscanf(line, "%599s %u %u %f %u %u %u %llu", key, &w, &ew, &lf, &dg, &team, &ol, &hc);
        if (got >= 6 && sig == key) {
            cfg.open_list = got >= 7 ? ol : 0;
            if (got == 8 && hc) cfg.heavy_cells = hc;
            cfg.warps_per_block = w;
            cfg.expansion_width = ew;
            cfg.load_factor = lf;
            cfg.delta_grid = dg;
            cfg.heavy_team = team;
            found = true;  // the last matching line wins
        }
    }
    std::fclose(f);
    return found;
}

// Estimated device time of the full batch from one trial batch over `idx`
// with configuration `cfg`.  The sample's persistent launch runs on the same
// share of the GPU as the sample is of the batch, so that blocks per instance
// -- which decides whether teams pay -- and the launch's time match the full
// run.  Its overflow re-runs and plain re-solves use the whole GPU, as they do
// in the full run, where there are 1 / share times as many of them: that part
// is scaled up accordingly (a configuration that overflows more is not
// favoured because the sample has few overflows).
int trial(gastar_batch* b, const std::vector<uint32_t>& idx, const gastar_batch_config& cfg, float& ms) {
    gastar_batch* t = gastar_batch_create(b->ctx, &cfg);
    if (!t) return GASTAR_OUT_OF_MEMORY;
    t->cfg.use_graph = 0;
    const double share = std::min(1.0, (double)idx.size() / (double)b->insts.size());
    t->block_share = share;
    for (uint32_t i : idx) t->insts.push_back(b->insts[i]);
    const int rc = gastar_batch_run(t);
    const double after = (double)t->retry_ms + (double)t->promote_ms;
    ms = (float)((double)t->kernel_ms - after + after / share);
    for (uint32_t j = 0; rc == GASTAR_OK && j < idx.size(); ++j)
        if (t->h_ctl[j].status != ST_OK && t->h_ctl[j].status != ST_NO_PATH) ms = 1e30f;  // unusable
    gastar_batch_destroy(t);
    return rc;
}

}  // namespace

extern "C" int gastar_batch_autotune(gastar_batch* b, uint32_t sample, const char* cache_path,
                                     gastar_batch_config* out, float* best_ms) {
    if (!b || b->uploaded || b->insts.empty()) return GASTAR_BAD_INPUT;
    const std::string sig = mix_signature(b);
    gastar_batch_config best = b->cfg;
    if (cache_lookup(cache_path, sig, best)) {
        b->cfg = best;
        if (out) *out = best;
        if (best_ms) *best_ms = 0.f;
        return GASTAR_OK;
    }
    // Stratified sample: every k-th instance in estimated-work order.
    std::vector<uint32_t> all(b->insts.size());
    std::iota(all.begin(), all.end(), 0u);
    std::stable_sort(all.begin(), all.end(),
                     [&](uint32_t x, uint32_t y) { return b->insts[x].est > b->insts[y].est; });
    const uint32_t m = std::max(1u, std::min<uint32_t>(sample ? sample : 64, (uint32_t)all.size()));
    std::vector<uint32_t> idx;
    for (uint32_t j = 0; j < m; ++j) idx.push_back(all[(size_t)j * all.size() / m]);
    bool grids = false, heavy = false;
    for (uint32_t i : idx) {
        grids |= b->insts[i].kind == KIND_GRID;
        heavy |= b->insts[i].kind == KIND_GRID &&
                 (uint64_t)b->insts[i].W * b->insts[i].H >= b->cfg.heavy_cells;
    }
    float best_t = 0;
    int rc = trial(b, idx, best, best_t);
    if (rc != GASTAR_OK) return rc;
    auto try_values = [&](auto setter, std::initializer_list<double> values) -> int {
        for (double v : values) {
            gastar_batch_config c = best;
            setter(c, v);
            if (std::memcmp(&c, &best, sizeof(c)) == 0) continue;
            float t = 0;
            const int r = trial(b, idx, c, t);
            if (r == GASTAR_OUT_OF_MEMORY) continue;
            if (r != GASTAR_OK) return r;
            if (t < best_t) {
                best_t = t;
                best = c;
            }
        }
        return GASTAR_OK;
    };
    if ((rc = try_values([](gastar_batch_config& c, double v) { c.open_list = (uint32_t)v; }, {0, 1})) !=
        GASTAR_OK)
        return rc;
    if ((rc = try_values([](gastar_batch_config& c, double v) { c.warps_per_block = (uint32_t)v; },
                         {4, 8, 16})) != GASTAR_OK)
        return rc;
    if ((rc = try_values([](gastar_batch_config& c, double v) { c.expansion_width = (uint32_t)v; },
                         {16, 32})) != GASTAR_OK)
        return rc;
    if (grids && (rc = try_values([](gastar_batch_config& c, double v) { c.delta_grid = (uint32_t)v; },
                                  {9, 12, 18, 36})) != GASTAR_OK)
        return rc;
    if (heavy && (rc = try_values([](gastar_batch_config& c, double v) { c.heavy_team = (uint32_t)v; },
                                  {1, 2, 4, 8})) != GASTAR_OK)
        return rc;
    if (heavy && best.heavy_team > 1 &&
        (rc = try_values([](gastar_batch_config& c, double v) { c.heavy_cells = (uint64_t)v; },
                         {(double)(1u << 20), (double)(1u << 21), (double)(1u << 22)})) != GASTAR_OK)
        return rc;
    // The pop window again under the chosen teams: with two-block teams on the
    // batched mix windows 9 and 12 tie, with one-block grids 9 is ~10 % faster.
    if (grids && heavy &&
        (rc = try_values([](gastar_batch_config& c, double v) { c.delta_grid = (uint32_t)v; },
                         {9, 12, 18})) != GASTAR_OK)
        return rc;
    if ((rc = try_values([](gastar_batch_config& c, double v) { c.load_factor = (float)v; },
                         {0.5, 0.7, 0.85})) != GASTAR_OK)
        return rc;
    b->cfg = best;
    if (cache_path) {
        if (FILE* f = std::fopen(cache_path, "a")) {
            std::fprintf(f, "%s %u %u %.3f %u %u %u %llu\n", sig.c_str(), best.warps_per_block, best.expansion_width,
                         best.load_factor, best.delta_grid, best.heavy_team, best.open_list,
                         (unsigned long long)best.heavy_cells);
            std::fclose(f);
        }
    }
    if (out) *out = best;
    if (best_ms) *best_ms = best_t;
    return GASTAR_OK;
}
