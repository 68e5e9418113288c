// Served GA*: a continuous-batching request loop.
//
// Requests (puzzles or grids) wait in a FIFO queue.  Each scheduling round
// (gastar_serve_step) admits waiting requests while a device slot and enough
// of the device-memory budget are free (partitions come from one arena of
// `budget_bytes` through a first-fit allocator), then runs one persistent
// launch over every active request for at most `slice_iters` GA* iterations
// each.  The search state (table, warp-heaps, control block) stays resident
// between rounds; finished requests get their path rebuilt, release their
// partition and slot, and the next round admits new work into them.  So
// requests that arrive while others are on the GPU join as capacity frees up,
// and their iterations interleave with the running ones inside the same
// launches.  A request whose partition overflows is re-queued at the front
// with 4x larger partitions.
//
// The reference has no counterpart: it solves one instance per process.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <unordered_map>
#include <vector>

#include "../../include/gastar.h"
#include "device_common.cuh"
#include "engine_internal.h"
#include "partition.h"

using namespace gastar;
using Clock = std::chrono::steady_clock;

namespace {

// First-fit allocator over [0, size) with coalescing of free ranges.
struct RangeAlloc {
    std::map<uint64_t, uint64_t> free_;  // offset -> length
    uint64_t in_use = 0;
    void reset(uint64_t size) {
        free_.clear();
        if (size) free_[0] = size;
        in_use = 0;
    }
    bool alloc(uint64_t n, uint64_t& off) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            off = it->first;
            const uint64_t rest = it->second - n;
            free_.erase(it);
            if (rest) free_[off + n] = rest;
            in_use += n;
            return true;
        }
        return false;
    }
    void release(uint64_t off, uint64_t n) {
        in_use -= n;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
};

enum ReqState { WAITING = 0, ACTIVE = 1, DONE = 2 };

struct Request {
    Problem prob;
    bool heavy = false;  // runs on a multi-block team
    uint32_t retry_level = 0;
    int state = WAITING;
    int slot = -1;
    uint64_t part_off = 0, part_bytes = 0;
    Clock::time_point t_submit, t_done;
    InstCtl ctl{};
    uint64_t prior_expansions = 0;
    uint32_t prior_iterations = 0;
    uint64_t w_off = 0, w_bytes = 0;  // grid weights placed in the weights pool at submission
    uint64_t exp_seen = 0;            // expansions in the current partition after the last step
    std::vector<unsigned long long> path;  // goal first
};

}  // namespace

struct gastar_server {
    gastar_ctx* ctx = nullptr;
    gastar_serve_config cfg;
    DevBuf arena, descs, ctls, order, counters, path_descs, path_arena, team_ctl, team_stage;
    // Grid weights of submitted requests, copied from the caller's buffer at
    // submission (an eighth of the budget, outside it; a host copy when full).
    DevBuf wpool;
    RangeAlloc walloc;
    uint32_t heavy_teams = 0;   // team buffers allocated (the most teams a launch can hold)
    uint32_t resident = 0;      // blocks resident on the device at once
    uint64_t heavy_stage_bytes = 0;
    uint32_t heap_snodes = kHeapSmemNodes;  // shared-memory heap nodes per warp
    RangeAlloc alloc;  // the arena
    uint32_t max_active = 0, threads = 0;
    size_t smem = 0;
    std::vector<InstDesc> h_desc;
    std::vector<int64_t> slot_req;
    std::vector<int> free_slots;
    InstCtl* h_ctl = nullptr;  // pinned, max_active
    std::deque<int64_t> waiting;
    std::unordered_map<int64_t, Request> reqs;
    int64_t next_id = 0;
    uint64_t completed = 0;
    uint64_t promoted = 0;  // puzzle requests finished by the plain engine
    float kernel_ms = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
};

namespace {

PartConfig serve_part_config(const gastar_server* s, uint32_t retry_level, bool heavy, bool own_weights) {
    PartConfig pc;
    pc.warps = s->cfg.warps_per_block * (heavy ? s->cfg.heavy_team : 1);
    pc.ew = s->cfg.expansion_width;
    pc.load_factor = s->cfg.load_factor;
    pc.heuristic = s->cfg.heuristic;
    pc.moves = s->cfg.moves;
    pc.delta_grid = s->cfg.delta_grid;
    pc.sliding_states = s->cfg.sliding_states;
    pc.retry_level = retry_level;
    pc.own_weights = own_weights;
    pc.heap_snodes = s->heap_snodes;
    pc.buckets = s->cfg.open_list == 1;
    return pc;
}

void finish_request(gastar_server* s, Request& r, const InstCtl& c) {
    r.ctl = c;
    r.ctl.expansions += r.prior_expansions;
    r.ctl.iterations += r.prior_iterations;
    r.state = DONE;
    r.t_done = Clock::now();
    ++s->completed;
    if (r.w_bytes) {  // weights placed at submission
        s->walloc.release(r.w_off, r.w_bytes);
        r.w_bytes = 0;
        r.prob.d_weights = nullptr;
    }
}

int64_t submit(gastar_server* s, Problem&& p, Clock::time_point t0, uint64_t w_off = 0, uint64_t w_bytes = 0) {
    const int64_t id = s->next_id++;
    Request r;
    r.prob = std::move(p);
    r.t_submit = t0;
    r.w_off = w_off;
    r.w_bytes = w_bytes;
    r.heavy = s->heavy_teams && r.prob.kind == KIND_GRID &&
              (uint64_t)r.prob.W * r.prob.H >= s->cfg.heavy_cells;
    if (r.prob.unreachable) {
        InstCtl c{};
        c.status = ST_NO_PATH;
        c.life = LIFE_DONE;
        auto& ref = s->reqs.emplace(id, std::move(r)).first->second;
        finish_request(s, ref, c);
        return id;
    }
    s->reqs.emplace(id, std::move(r));
    s->waiting.push_back(id);
    return id;
}

// Admits waiting requests in arrival order while a slot and memory are free.
// With admit_bypass set, a request that needs at most 1/256 of the budget
// (puzzles, small grids) may go ahead of a larger one that waits for memory;
// larger requests keep their arrival order among themselves, so the one at
// the head is not passed by another large one.
int admit(gastar_server* s, cudaStream_t st) {
    const uint64_t small = s->cfg.admit_bypass ? s->arena.n / 256 : 0;
    bool blocked = false;  // a request larger than `small` waits for memory
    for (auto it = s->waiting.begin(); it != s->waiting.end() && !s->free_slots.empty();) {
        const int64_t id = *it;
        Request& r = s->reqs[id];
        const bool own = r.prob.kind == KIND_GRID && !r.prob.d_weights;
        const PartConfig pc = serve_part_config(s, r.retry_level, r.heavy, own);
        const PartPlan plan = plan_partition(r.prob, pc);
        if (plan.bytes > s->arena.n) {  // can never fit the budget
            it = s->waiting.erase(it);
            InstCtl c{};
            c.status = GASTAR_OUT_OF_MEMORY;
            c.life = LIFE_DONE;
            finish_request(s, r, c);
            continue;
        }
        if (blocked && plan.bytes > small) {
            ++it;
            continue;
        }
        uint64_t off;
        if (!s->alloc.alloc(plan.bytes, off)) {  // wait for memory to free up
            if (!small) break;
            blocked = true;
            ++it;
            continue;
        }
        it = s->waiting.erase(it);
        const int slot = s->free_slots.back();
        s->free_slots.pop_back();
        r.slot = slot;
        r.part_off = off;
        r.part_bytes = plan.bytes;
        r.exp_seen = 0;
        r.state = ACTIVE;
        s->slot_req[slot] = id;
        char* base = reinterpret_cast<char*>(s->arena.p) + off;
        InstCtl* ctl = reinterpret_cast<InstCtl*>(s->ctls.p) + slot;
        fill_desc(s->h_desc[slot], r.prob, pc, plan, base, r.prob.d_weights, ctl);
        if (own &&
            !cuda_ok(cudaMemcpyAsync(base + plan.weights_off, r.prob.weights.data(), r.prob.weights.size(),
                                     cudaMemcpyHostToDevice, st), "cudaMemcpyAsync"))
            return GASTAR_CUDA_ERROR;
        if (!cuda_ok(cudaMemsetAsync(ctl, 0, sizeof(InstCtl), st), "cudaMemsetAsync") ||
            !cuda_ok(cudaMemcpyAsync(reinterpret_cast<InstDesc*>(s->descs.p) + slot, &s->h_desc[slot],
                                     sizeof(InstDesc), cudaMemcpyHostToDevice, st), "cudaMemcpyAsync"))
            return GASTAR_CUDA_ERROR;
    }
    return GASTAR_OK;
}

// A hard puzzle request leaves the time-sliced launches: the plain engine
// finishes it on the whole GPU (65536 parallel pops, a 2^26-slot table) and
// its partition is released.  A puzzle that runs for millions of expansions
// on one block holds its slot for seconds; the plain engine takes a few
// milliseconds.
int promote(gastar_server* s, Request& r, const InstCtl& sofar) {
    PlainProblem pp;
    std::memset(&pp, 0, sizeof(pp));
    pp.kind = r.prob.kind;
    pp.n = r.prob.n;
    pp.start0 = r.prob.start0;
    pp.start1 = r.prob.start1;
    pp.goal0 = r.prob.goal0;
    pp.goal1 = r.prob.goal1;
    pp.f0 = r.prob.f0;
    gastar_config cfg;
    gastar_config_default(&cfg);
    cfg.num_queues = 65536;
    cfg.heuristic = s->cfg.heuristic;
    cfg.moves = s->cfg.moves;
    cfg.table_log2 = r.prob.kind == KIND_SLIDING5 ? 27 : 26;
    cfg.heap_entries = 1ull << 25;
    std::vector<uint64_t> keys;
    gastar_result res;
    std::memset(&res, 0, sizeof(res));
    const int rc = plain_solve(s->ctx, pp, &cfg, &keys, &res);
    if (rc != GASTAR_OK) return rc;
    InstCtl c = sofar;
    c.life = LIFE_DONE;
    c.status = (uint32_t)res.status;
    c.best = res.cost;
    c.path_len = res.status == GASTAR_OK ? res.path_len : 0;
    c.iterations += res.iterations;
    c.expansions += res.expansions;
    c.generated += res.generated;
    c.pushes += res.pushes;
    c.stale += res.stale;
    c.table_used = res.table_used;
    if (res.status == GASTAR_OK) r.path.assign(keys.begin(), keys.end());
    s->kernel_ms += res.kernel_ms;
    ++s->promoted;
    finish_request(s, r, c);
    return GASTAR_OK;
}

void release_slot(gastar_server* s, Request& r) {
    s->alloc.release(r.part_off, r.part_bytes);
    s->slot_req[r.slot] = -1;
    s->free_slots.push_back(r.slot);
    r.slot = -1;
}

}  // namespace

extern "C" {

void gastar_serve_config_default(gastar_serve_config* c) {
    std::memset(c, 0, sizeof(*c));
    c->budget_bytes = 120ull << 30;
    // 128 iterations per slice: burst capacity 205 req/s against 196 with 64
    // and 204 with 256 (fewer steps, each with its own host round trip).
    c->slice_iters = 128;
    c->warps_per_block = 8;
    c->expansion_width = 32;
    c->load_factor = 0.75f;
    // Pop window 8 for grids: on the served mix's large grids (eight-block
    // teams) it gave 133-140 req/s of burst capacity against 122-131 with 18
    // and a shorter longest grid (3.2 against 3.6-3.9 s); 4 and 6 were slower.
    c->delta_grid = 8;
    c->heavy_team = 8;  // the largest grids (8192^2) bound the tail latency
    c->heavy_cells = 1ull << 20;
    c->open_list = 1;
    // Promotion past 2^18 expansions: under Poisson arrivals at 110 req/s of
    // the served mix, 15-puzzle p99 34 ms and overall p99 0.74 s, against
    // 0.5 s and 1.15 s past 2^21; burst capacity unchanged (156-164 req/s).
    c->promote_log2 = 18;
    c->admit_bypass = 1;
    c->weights_pool = 1;
    c->weighted_slices = 1;
    c->heavy_set = 4;
}

gastar_server* gastar_serve_create(gastar_ctx* c, const gastar_serve_config* cfg) {
    if (!c) return nullptr;
    if (cudaSetDevice(c->device) != cudaSuccess) return nullptr;
    auto* s = new gastar_server();
    s->ctx = c;
    if (cfg) s->cfg = *cfg;
    else gastar_serve_config_default(&s->cfg);
    auto& cf = s->cfg;
    if (!cf.warps_per_block) cf.warps_per_block = 8;
    cf.warps_per_block = std::min(16u, cf.warps_per_block);
    if (!cf.expansion_width) cf.expansion_width = 32;
    cf.expansion_width = std::min(32u, cf.expansion_width);
    if (cf.load_factor <= 0.f) cf.load_factor = 0.75f;
    if (!cf.slice_iters) cf.slice_iters = 128;
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    uint64_t budget = cf.budget_bytes ? cf.budget_bytes : (120ull << 30);
    budget = std::min<uint64_t>(budget, free_b > (2ull << 30) ? free_b - (2ull << 30) : free_b / 2);
    cf.budget_bytes = budget;
    s->threads = cf.warps_per_block * 32;
    const bool buckets = cf.open_list == 1;
    s->smem = block_smem_bytes(kKindsAll, cf.warps_per_block, cf.expansion_width, false, kHeapSmemNodes, buckets);
    if (s->smem + 4096 > c->smem_optin) {  // + the kernel's static shared memory
        set_error("serve: warps_per_block x expansion_width needs more shared memory than a block has");
        delete s;
        return nullptr;
    }
    const int nb = occupancy_blocks(c, kKindsAll, s->threads, s->smem);
    if (nb <= 0) {
        delete s;
        return nullptr;
    }
    s->heap_snodes = fit_heap_snodes(c, kKindsAll, cf.warps_per_block, cf.expansion_width, false, s->threads, nb,
                                     &s->smem, buckets);
    const uint32_t resident = (uint32_t)(nb * c->sms);
    s->resident = resident;
    s->max_active = cf.max_active ? cf.max_active : resident;
    const uint32_t m = s->max_active;
    if (!cf.heavy_team) cf.heavy_team = 1;
    if (cf.heavy_team > 1) {
        // Buffers for as many teams as the resident blocks hold; each step
        // uses as many as its heavy requests and the light ones leave room for.
        s->heavy_teams = cf.heavy_teams ? cf.heavy_teams : resident / cf.heavy_team;
        s->heavy_teams = std::min(s->heavy_teams, resident / cf.heavy_team);
        s->heavy_stage_bytes = team_stage_bytes(cf.heavy_team, cf.warps_per_block, cf.expansion_width, 8, 16);
        if (!s->heavy_teams || !s->team_ctl.ensure(sizeof(TeamCtl) * s->heavy_teams) ||
            !s->team_stage.ensure(s->heavy_stage_bytes * s->heavy_teams))
            s->heavy_teams = 0;
    }
    if (!s->arena.ensure(budget) || !s->descs.ensure(sizeof(InstDesc) * m) ||
        !s->ctls.ensure(sizeof(InstCtl) * m) || !s->order.ensure(2 * sizeof(uint32_t) * m) ||
        !s->counters.ensure(64) ||
        !cuda_ok(cudaMallocHost(&s->h_ctl, sizeof(InstCtl) * m), "cudaMallocHost")) {
        gastar_serve_destroy(s);
        return nullptr;
    }
    s->alloc.reset(s->arena.n);
    {
        size_t f2 = 0, t2 = 0;
        cudaMemGetInfo(&f2, &t2);
        const uint64_t want = std::min<uint64_t>(budget / 8, f2 > (4ull << 30) ? f2 - (4ull << 30) : 0);
        if (cf.weights_pool && want >= (16ull << 20) && s->wpool.ensure(want)) {
            s->walloc.reset(s->wpool.n);
        } else {  // no pool: grids keep host copies
            cudaGetLastError();
            s->wpool.release();
        }
    }
    s->h_desc.assign(m, InstDesc());
    s->slot_req.assign(m, -1);
    for (int i = (int)m - 1; i >= 0; --i) s->free_slots.push_back(i);
    cudaEventCreate(&s->e0);
    cudaEventCreate(&s->e1);
    return s;
}

void gastar_serve_destroy(gastar_server* s) {
    if (!s) return;
    cudaSetDevice(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    s->arena.release();
    s->descs.release();
    s->ctls.release();
    s->order.release();
    s->counters.release();
    s->path_descs.release();
    s->path_arena.release();
    s->team_ctl.release();
    s->team_stage.release();
    s->wpool.release();
    if (s->h_ctl) cudaFreeHost(s->h_ctl);
    if (s->e0) cudaEventDestroy(s->e0);
    if (s->e1) cudaEventDestroy(s->e1);
    delete s;
}

int64_t gastar_serve_submit_sliding(gastar_server* s, uint32_t n, const uint8_t* start, const uint8_t* goal) {
    if (!s) return -GASTAR_BAD_INPUT;
    Problem p;
    const Clock::time_point t0 = Clock::now();
    if (!make_sliding_problem(n, start, goal, s->cfg.heuristic, s->cfg.moves, p)) {
        set_error("sliding: boards must be permutations of 0..n*n-1 with n in 3..5");
        return -GASTAR_BAD_INPUT;
    }
    return submit(s, std::move(p), t0);
}

int64_t gastar_serve_submit_grid(gastar_server* s, uint32_t w, uint32_t h, const uint8_t* weights,
                                 uint32_t sx, uint32_t sy, uint32_t tx, uint32_t ty) {
    if (!s) return -GASTAR_BAD_INPUT;
    const Clock::time_point t0 = Clock::now();
    Problem p;
    if (!make_grid_problem(w, h, weights, sx, sy, tx, ty, s->cfg.heuristic, p, false)) {
        set_error("grid: bad dimensions or endpoints");
        return -GASTAR_BAD_INPUT;
    }
    // The weights go from the caller's buffer to the weights pool and their
    // least passable weight is reduced there (a host copy's first-touch page
    // faults cost more than the transfer); a full pool keeps a host copy,
    // copied at admission.
    const uint64_t cells = (uint64_t)w * h, wb = (cells + 255) & ~255ull;
    uint64_t off = 0;
    if (s->wpool.n && s->walloc.alloc(wb, off)) {
        if (cudaSetDevice(s->ctx->device) != cudaSuccess) return -GASTAR_CUDA_ERROR;
        cudaStream_t st = s->ctx->stream;
        uint8_t* d = reinterpret_cast<uint8_t*>(s->wpool.p) + off;
        uint32_t mw = 255;
        const int rc = upload_grid(s->ctx, d, weights, cells, st, &mw);
        if (rc != GASTAR_OK) {
            s->walloc.release(off, wb);
            return -rc;
        }
        set_grid_minw(p, mw, s->cfg.heuristic);
        p.d_weights = d;
        return submit(s, std::move(p), t0, off, wb);
    }
    p.weights.assign(weights, weights + cells);
    set_grid_minw(p, min_passable_weight(weights, cells), s->cfg.heuristic);
    return submit(s, std::move(p), t0);
}

int gastar_serve_step(gastar_server* s) {
    if (!s) return GASTAR_BAD_INPUT;
    if (cudaSetDevice(s->ctx->device) != cudaSuccess) return GASTAR_CUDA_ERROR;
    cudaStream_t st = s->ctx->stream;
    int rc = admit(s, st);
    if (rc != GASTAR_OK) return rc;
    std::vector<uint32_t> active, light, heavy;
    for (uint32_t i = 0; i < s->max_active; ++i)
        if (s->slot_req[i] >= 0) {
            active.push_back(i);
            (s->reqs[s->slot_req[i]].heavy ? heavy : light).push_back(i);
        }
    if (active.empty()) return GASTAR_OK;
    // Longest work first inside the launch (sched_before); the order array
    // holds the one-block requests, then the heavy ones.
    auto by_est = [&](uint32_t a, uint32_t b) {
        return sched_before(s->reqs[s->slot_req[a]].prob, s->reqs[s->slot_req[b]].prob);
    };
    std::stable_sort(light.begin(), light.end(), by_est);
    std::stable_sort(heavy.begin(), heavy.end(), by_est);
    // Teams the launch can hold: one-block requests keep up to a quarter of
    // the resident blocks (as many as there are of them), heavy requests get
    // the rest in teams.
    const uint32_t reserve = std::min<uint32_t>((uint32_t)light.size(), s->resident / 4);
    const uint32_t team_cap =
        std::min(std::max(1u, (s->resident - reserve) / std::max(1u, s->cfg.heavy_team)), s->heavy_teams);
    // The order array (one-block requests, then heavy ones), then, at the end
    // of a burst -- nothing but heavy requests left, more of them than teams,
    // so that teams take turns -- a slice length per slot: 1/2x to 4x the
    // configured slice in proportion to each request's estimated work left
    // (its one-block estimate less ~100 ns per expansion done), so that the
    // largest grids do not all finish last, each on its own team while the
    // other teams idle.  With a team per request, equal slices keep every
    // team busy until the launch ends.
    std::vector<uint32_t> order(light.size() + heavy.size() + s->max_active);
    std::copy(light.begin(), light.end(), order.begin());
    std::copy(heavy.begin(), heavy.end(), order.begin() + light.size());
    const uint32_t n = (uint32_t)(light.size() + heavy.size());
    bool weighted = false;
    if (s->cfg.weighted_slices && light.empty() && s->waiting.empty() && heavy.size() > team_cap) {
        std::vector<uint64_t> left(heavy.size());
        for (size_t k = 0; k < heavy.size(); ++k) {
            const Request& r = s->reqs[s->slot_req[heavy[k]]];
            const uint64_t done = 100ull * (r.prior_expansions + r.exp_seen);
            left[k] = std::max<uint64_t>(r.prob.est > done ? r.prob.est - done : 0, r.prob.est / 16 + 1);
        }
        std::vector<uint64_t> sorted(left);
        std::nth_element(sorted.begin(), sorted.begin() + sorted.size() / 2, sorted.end());
        const double med = (double)sorted[sorted.size() / 2];
        const uint32_t base = s->cfg.slice_iters;
        uint32_t* sl = order.data() + n;
        for (uint32_t i = 0; i < s->max_active; ++i) sl[i] = base;
        for (size_t k = 0; k < heavy.size(); ++k)
            sl[heavy[k]] = (uint32_t)std::min(4.0 * base, std::max(0.5 * base, base * (double)left[k] / med));
        weighted = true;
    }
    if (!cuda_ok(cudaMemcpyAsync(s->order.p, order.data(), 4ull * (weighted ? n + s->max_active : n),
                                 cudaMemcpyHostToDevice, st),
                 "cudaMemcpyAsync") ||
        !cuda_ok(cudaMemsetAsync(s->counters.p, 0, 32, st), "cudaMemsetAsync"))
        return GASTAR_CUDA_ERROR;
    LaunchParams P;
    std::memset(&P, 0, sizeof(P));
    P.insts = reinterpret_cast<const InstDesc*>(s->descs.p);
    P.n_insts = (uint32_t)light.size();
    P.heap_snodes = s->heap_snodes;
    P.buckets = s->cfg.open_list == 1 ? 1u : 0u;
    P.order = reinterpret_cast<const uint32_t*>(s->order.p);
    P.next = reinterpret_cast<uint32_t*>(s->counters.p);
    P.team_ctas = 1;
    P.slice_iters = s->cfg.slice_iters;
    P.slices = weighted ? reinterpret_cast<const uint32_t*>(s->order.p) + n : nullptr;
    P.barrier_timeout_ns = 2000000000ull;
    uint32_t blocks = std::min((uint32_t)light.size(), s->max_active);
    if (!heavy.empty()) {
        // Team blocks that run out of heavy requests take one-block requests,
        // and every block of the launch is resident (a cooperative launch),
        // so a team's blocks always run together.
        const uint32_t T = s->cfg.heavy_team;
        const uint32_t teams = std::min(team_cap, (uint32_t)heavy.size());
        blocks = std::min(s->resident, teams * T + (uint32_t)light.size());
        P.heavy_order = reinterpret_cast<const uint32_t*>(s->order.p) + light.size();
        // At most heavy_set x teams heavy requests, the largest first, take
        // turns in a launch: fewer grids per launch keep their frontiers in
        // L2 between slices (burst capacity 267 against 252 req/s with all;
        // 2x the teams: 226, 3x: 251, 6x: 257); the teams still share them
        // dynamically, and the rest run as the largest finish.
        P.n_heavy = (uint32_t)heavy.size();
        if (s->cfg.heavy_set)
            P.n_heavy = (uint32_t)std::min<uint64_t>(heavy.size(), (uint64_t)s->cfg.heavy_set * teams);
        P.heavy_team = s->cfg.heavy_team;
        P.heavy_teams = teams;
        P.heavy_next = reinterpret_cast<uint32_t*>(s->counters.p) + 4;
        P.heavy_ctl = reinterpret_cast<TeamCtl*>(s->team_ctl.p);
        P.heavy_stage = s->team_stage.p;
        P.heavy_stage_bytes = s->heavy_stage_bytes;
        if (!cuda_ok(cudaMemsetAsync(s->team_ctl.p, 0, sizeof(TeamCtl) * teams, st), "cudaMemsetAsync"))
            return GASTAR_CUDA_ERROR;
    }
    cudaEventRecord(s->e0, st);
    rc = launch_search(s->ctx, kKindsAll, P, blocks, s->threads, s->smem, st);
    if (rc != GASTAR_OK) return rc;
    cudaEventRecord(s->e1, st);
    if (!cuda_ok(cudaMemcpyAsync(s->h_ctl, s->ctls.p, sizeof(InstCtl) * s->max_active,
                                 cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync") ||
        !cuda_ok(cudaStreamSynchronize(st), "cudaStreamSynchronize"))
        return GASTAR_CUDA_ERROR;
    float ms = 0;
    cudaEventElapsedTime(&ms, s->e0, s->e1);
    s->kernel_ms += ms;

    // Retire finished requests: paths for the solved ones, re-queue overflows.
    std::vector<uint32_t> solved;
    std::vector<int64_t> requeue;
    for (uint32_t slot : active) {
        const InstCtl& c = s->h_ctl[slot];
        Request& r = s->reqs[s->slot_req[slot]];
        r.exp_seen = c.expansions;
        if (c.life != LIFE_DONE) {
            const uint32_t pl = s->cfg.promote_log2;
            if (pl && pl < 64 && r.prob.kind != KIND_GRID && r.prob.n >= 4 &&
                c.expansions + r.prior_expansions > (1ull << pl)) {
                rc = promote(s, r, c);
                if (rc != GASTAR_OK) return rc;
                release_slot(s, r);
            }
            continue;
        }
        if ((c.status == ST_TABLE_FULL || c.status == ST_HEAP_FULL) && r.retry_level < 3) {
            r.prior_expansions += c.expansions;
            r.prior_iterations += c.iterations;
            r.retry_level += 1;
            r.state = WAITING;
            requeue.push_back(s->slot_req[slot]);
            release_slot(s, r);
            continue;
        }
        if (c.status == ST_OK) solved.push_back(slot);
        else {
            finish_request(s, r, c);
            release_slot(s, r);
        }
    }
    for (auto it = requeue.rbegin(); it != requeue.rend(); ++it) s->waiting.push_front(*it);
    if (!solved.empty()) {
        // Descriptors, then each path's slice of the arena (best + 1 states
        // at most, every step lowering g by at least 1), in one upload: the
        // paths are written in a single walk each.
        const uint32_t m = (uint32_t)solved.size();
        const size_t desc_bytes = (sizeof(InstDesc) * m + 7) & ~size_t(7);
        std::vector<unsigned char> up(desc_bytes + 8 * (size_t)(m + 1));
        unsigned long long* offs = reinterpret_cast<unsigned long long*>(up.data() + desc_bytes);
        uint64_t words = 0;
        for (uint32_t k = 0; k < m; ++k) {
            const uint32_t slot = solved[k];
            std::memcpy(up.data() + sizeof(InstDesc) * k, &s->h_desc[slot], sizeof(InstDesc));
            offs[k] = words;
            words += ((uint64_t)s->h_ctl[slot].best + 2) * key_words(s->h_desc[slot].kind);
        }
        offs[m] = words;
        if (!s->path_descs.ensure(up.size()) || !s->path_arena.ensure(words * 8 + 16))
            return GASTAR_OUT_OF_MEMORY;
        unsigned long long* used = reinterpret_cast<unsigned long long*>(s->counters.p) + 2;
        if (!cuda_ok(cudaMemcpyAsync(s->path_descs.p, up.data(), up.size(), cudaMemcpyHostToDevice, st),
                     "cudaMemcpyAsync") ||
            !cuda_ok(cudaMemsetAsync(used, 0, 8, st), "cudaMemsetAsync"))
            return GASTAR_CUDA_ERROR;
        rc = launch_paths(reinterpret_cast<const InstDesc*>(s->path_descs.p), m,
                          reinterpret_cast<unsigned long long*>(s->path_arena.p), words, used, st,
                          reinterpret_cast<const unsigned long long*>(
                              reinterpret_cast<const char*>(s->path_descs.p) + desc_bytes));
        if (rc != GASTAR_OK) return rc;
        std::vector<unsigned long long> arena(words);
        if (!cuda_ok(cudaMemcpyAsync(s->h_ctl, s->ctls.p, sizeof(InstCtl) * s->max_active,
                                     cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync") ||
            !cuda_ok(cudaMemcpyAsync(arena.data(), s->path_arena.p, words * 8, cudaMemcpyDeviceToHost, st),
                     "cudaMemcpyAsync") ||
            !cuda_ok(cudaStreamSynchronize(st), "cudaStreamSynchronize"))
            return GASTAR_CUDA_ERROR;
        for (uint32_t slot : solved) {
            const InstCtl& c = s->h_ctl[slot];
            Request& r = s->reqs[s->slot_req[slot]];
            if (c.status == ST_OK) {
                const uint64_t w = (uint64_t)c.path_len * key_words(r.prob.kind);
                r.path.assign(arena.begin() + c.path_off, arena.begin() + c.path_off + w);
            }
            finish_request(s, r, c);
            release_slot(s, r);
        }
    }
    return GASTAR_OK;
}

int gastar_serve_poll(gastar_server* s, int64_t id, gastar_result* out, void* path, uint32_t cap,
                      uint32_t* len) {
    if (!s || !out) return GASTAR_BAD_INPUT;
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return GASTAR_BAD_INPUT;
    const Request& r = it->second;
    std::memset(out, 0, sizeof(*out));
    if (r.state != DONE) {
        out->status = GASTAR_PENDING;
        return GASTAR_PENDING;
    }
    const InstCtl& c = r.ctl;
    out->status = (int32_t)c.status;
    out->cost = c.status == ST_OK ? c.best : 0;
    out->path_len = c.status == ST_OK ? c.path_len : 0;
    out->iterations = c.iterations;
    out->expansions = c.expansions;
    out->generated = c.generated;
    out->pushes = c.pushes;
    out->stale = c.stale;
    out->table_used = c.table_used;
    out->total_ms = std::chrono::duration<float, std::milli>(r.t_done - r.t_submit).count();
    out->attempts = 1 + r.retry_level;
    if (len) *len = out->path_len;
    if (path && c.status == ST_OK) {
        if (c.path_len > cap) return GASTAR_PATH_CAP;
        const uint32_t kw = key_words(r.prob.kind);
        for (uint32_t i = 0; i < c.path_len; ++i) {
            const uint32_t j = c.path_len - 1 - i;  // stored goal-first
            if (r.prob.kind == KIND_GRID) reinterpret_cast<uint32_t*>(path)[i] = (uint32_t)r.path[j];
            else
                unpack_board(r.prob.n, r.path[(size_t)j * kw], kw == 2 ? r.path[(size_t)j * kw + 1] : 0,
                             reinterpret_cast<uint8_t*>(path) + (size_t)i * r.prob.n * r.prob.n);
        }
    }
    return GASTAR_OK;
}

int gastar_serve_release(gastar_server* s, int64_t id) {
    if (!s) return GASTAR_BAD_INPUT;
    auto it = s->reqs.find(id);
    if (it == s->reqs.end() || it->second.state != DONE) return GASTAR_BAD_INPUT;
    s->reqs.erase(it);
    return GASTAR_OK;
}

int gastar_serve_stats(gastar_server* s, uint32_t* waiting, uint32_t* active, uint64_t* completed,
                       uint64_t* bytes_in_use, float* kernel_ms) {
    if (!s) return GASTAR_BAD_INPUT;
    if (waiting) *waiting = (uint32_t)s->waiting.size();
    if (active) *active = s->max_active - (uint32_t)s->free_slots.size();
    if (completed) *completed = s->completed;
    if (bytes_in_use) *bytes_in_use = s->alloc.in_use;
    if (kernel_ms) *kernel_ms = s->kernel_ms;
    return GASTAR_OK;
}

}  // extern "C"
