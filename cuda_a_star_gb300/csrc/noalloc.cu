// 8-puzzle solve that allocates nothing: gastar_solve_sliding_noalloc.
//
// Some callers cannot call cudaMalloc: a host program that has reserved all
// device memory for its own pool before loading this library, or a real-time
// loop that must not take the device-wide synchronisation cudaMalloc/cudaFree
// can cause.  For them this entry point runs the same search kernel as
// gastar_solve_sliding on a fixed scratch area that is part of the library
// image: a file-scope device array of kScratchBytes (about 16 MiB), which every
// GPU that loads the library holds until the process exits.  The caller passes
// the boards and the output buffers as for gastar_solve_sliding.
//
// Only 3x3 boards are accepted: the whole 8-puzzle state space (181,440
// states reachable from any board) fits the table in the array, so no solve
// can outgrow it.  Larger boards are rejected with GASTAR_BAD_INPUT.
//
// Every call uses the same array and the array keeps the previous call's
// contents; the search clears its table and control words itself.  Calls that
// overlap on the GPU (two host threads, or two streams) race on the array and
// must be serialised by the caller.  In host code the array's name is only a
// host-side stand-in, so every call looks up the array's device address with
// cudaGetSymbolAddress on the device that is current: the lookup resolves
// against the current context, so it stays right after a cudaDeviceReset.
// The call synchronises the stream it runs on before it returns.
#include <cuda_runtime.h>

#include <chrono>
#include <cstring>

#include "../../include/gastar.h"
#include "engine_internal.h"
#include "search.cuh"

namespace {

using namespace gastar;

constexpr uint32_t kWarps = 4;           // warp-heaps of the single block
constexpr uint32_t kEw = 32;             // pops per warp-heap per iteration
constexpr uint64_t kTableSlots = 1ull << 19;  // hash slots: 181,440 states at load 0.35
constexpr uint32_t kHeapCap = 4095;      // nodes per warp-heap (131,040 entries)
constexpr uint64_t kPathWords = 4096;    // path arena (states)

constexpr size_t kDescOff = 0;
constexpr size_t kCtlOff = 512;
constexpr size_t kNextOff = 640;         // u32 work counter
constexpr size_t kUsedOff = 648;         // u64 path-arena fill
constexpr size_t kHdrOff = 1024;         // kWarps x {N, pc}
constexpr size_t kPathOff = 4096;
constexpr size_t kTableOff = kPathOff + kPathWords * 8;
constexpr size_t kHeapOff = kTableOff + kTableSlots * 16;
constexpr size_t kScratchBytes = kHeapOff + (size_t)kWarps * (kHeapCap + 1) * 32 * 16;

static_assert(sizeof(InstDesc) <= kCtlOff - kDescOff, "descriptor does not fit");
static_assert(kCtlOff + sizeof(InstCtl) <= kNextOff, "control block does not fit");
static_assert(kTableOff % 256 == 0 && kHeapOff % 256 == 0, "alignment");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of the scratch array in the current context.  Looked up on
// every call: a cached address would go stale when the caller resets the
// device or destroys its primary context and the module is loaded again.
int scratch_for_current_device(void** out) {
    void* p = nullptr;
    if (!cuda_ok(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress"))
        return GASTAR_CUDA_ERROR;
    *out = p;
    return GASTAR_OK;
}

}  // namespace

extern "C" int gastar_solve_sliding_noalloc(uint32_t n, const uint8_t* start, const uint8_t* goal,
                                            const gastar_config* cfg, uint8_t* path, uint32_t path_cap,
                                            gastar_result* out) {
    const auto t0 = std::chrono::steady_clock::now();
    if (!out) return GASTAR_BAD_INPUT;
    std::memset(out, 0, sizeof(*out));
    if (n != 3) {
        set_error("gastar_solve_sliding_noalloc: only 3x3 boards fit the static scratch "
                  "(16 MiB, the whole 8-puzzle state space); use gastar_solve_sliding");
        out->status = GASTAR_BAD_INPUT;
        return GASTAR_BAD_INPUT;
    }
    if (!valid_board(n, start) || !valid_board(n, goal)) {
        set_error("sliding: boards must be permutations of 0..8");
        out->status = GASTAR_BAD_INPUT;
        return GASTAR_BAD_INPUT;
    }
    gastar_config dc;
    gastar_config_default(&dc);
    const gastar_config& cf = cfg ? *cfg : dc;
    auto finish = [&]() {
        out->total_ms =
            std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
        return GASTAR_OK;
    };
    if (cf.moves == GASTAR_MOVES_STANDARD && !sliding_solvable(n, start, goal)) {
        out->status = GASTAR_NO_PATH;
        return finish();
    }
    void* base = nullptr;
    int rc = scratch_for_current_device(&base);
    if (rc != GASTAR_OK) {
        out->status = rc;
        return rc;
    }
    char* b = static_cast<char*>(base);
    cudaStream_t st = cf.stream ? (cudaStream_t)cf.stream : (cudaStream_t)0;

    InstDesc d;
    std::memset(&d, 0, sizeof(d));
    d.kind = KIND_SLIDING3;
    d.heuristic = cf.heuristic;
    d.moves = cf.moves;
    d.n = 3;
    pack_board(3, start, d.start0, d.start1);
    pack_board(3, goal, d.goal0, d.goal1);
    d.f0 = sliding_h(3, start, goal, cf.heuristic);
    d.table = reinterpret_cast<unsigned long long*>(b + kTableOff);
    d.table_words = kTableSlots * 2;
    d.table_mask = kTableSlots - 1;
    d.table_limit = kTableSlots - kTableSlots / 8;
    d.max_probe = 4096;
    d.heaps = kWarps;
    d.heap_nodes = b + kHeapOff;
    d.heap_hdr = reinterpret_cast<uint32_t*>(b + kHdrOff);
    d.heap_cap = kHeapCap;
    d.ew = kEw;
    d.max_exp = cf.max_expansions;
    d.timeout_ns = (uint64_t)cf.timeout_ms * 1000000ull;
    d.max_iter = cf.max_iterations;
    d.delta = cf.delta;
    d.ctl = reinterpret_cast<InstCtl*>(b + kCtlOff);
    d.touched = nullptr;  // the kernel clears the whole table

    LaunchParams P;
    std::memset(&P, 0, sizeof(P));
    P.insts = reinterpret_cast<const InstDesc*>(b + kDescOff);
    P.n_insts = 1;
    P.next = reinterpret_cast<uint32_t*>(b + kNextOff);
    P.team_ctas = 1;
    P.barrier_timeout_ns = 2000000000ull;
    unsigned long long* used = reinterpret_cast<unsigned long long*>(b + kUsedOff);

    auto fail = [&](cudaError_t e, const char* what) {
        cuda_ok(e, what);
        out->status = GASTAR_CUDA_ERROR;
        return GASTAR_CUDA_ERROR;
    };
    cudaError_t e;
    if ((e = cudaMemcpyAsync(b + kDescOff, &d, sizeof(d), cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return fail(e, "cudaMemcpyAsync");
    // Control block, work counter and arena fill start at zero every call.
    if ((e = cudaMemsetAsync(b + kCtlOff, 0, kHdrOff - kCtlOff, st)) != cudaSuccess)
        return fail(e, "cudaMemsetAsync");
    out->h2d_bytes = sizeof(d);
    const void* kern = reinterpret_cast<const void*>(&search_kernel<kind_bit(KIND_SLIDING3)>);
    void* args[] = {&P};
    const size_t smem = 2 * stage_entries_per_buffer(kWarps, kEw, 4) * 16 + (size_t)kWarps * (kHeapSmemNodes - 1) * 32 * 16;
    if ((e = cudaLaunchKernel(kern, dim3(1), dim3(kWarps * 32), args, smem, st)) != cudaSuccess)
        return fail(e, "cudaLaunchKernel");
    out->launches = 1;
    InstCtl ctl;
    if ((e = cudaMemcpyAsync(&ctl, b + kCtlOff, sizeof(ctl), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return fail(e, "search");
    out->d2h_bytes = sizeof(ctl);
    if (ctl.status == ST_OK && path) {
        path_kernel<<<1, 32, 0, st>>>(P.insts, 1, reinterpret_cast<unsigned long long*>(b + kPathOff),
                                      kPathWords, used, nullptr);  // 8-puzzle: no grid window
        if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "path_kernel");
        out->launches = 2;
        if ((e = cudaMemcpyAsync(&ctl, b + kCtlOff, sizeof(ctl), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return fail(e, "path");
        out->d2h_bytes += sizeof(ctl);
    }
    if (ctl.status == ST_PATH_CAP && ctl.best != kInf) {
        // The goal was reached but its path is longer than the arena of
        // kPathWords states (possible only with the inadmissible heuristic):
        // the cost stands, the path is not returned.  Every move costs 1, so
        // the path needs best + 1 states.
        out->status = GASTAR_PATH_CAP;
        out->cost = ctl.best;
        out->path_len = ctl.best + 1;
        out->iterations = ctl.iterations;
        out->expansions = ctl.expansions;
        out->generated = ctl.generated;
        out->pushes = ctl.pushes;
        out->stale = ctl.stale;
        out->table_used = ctl.table_used;
        out->attempts = 1;
        return finish();
    }
    out->status = (int32_t)ctl.status;
    out->cost = ctl.status == ST_OK ? ctl.best : 0;
    out->path_len = ctl.path_len;
    out->iterations = ctl.iterations;
    out->expansions = ctl.expansions;
    out->generated = ctl.generated;
    out->pushes = ctl.pushes;
    out->stale = ctl.stale;
    out->table_used = ctl.table_used;
    out->attempts = 1;
    if (ctl.status == ST_OK && path) {
        if (ctl.path_len > path_cap) {
            out->status = GASTAR_PATH_CAP;
            return finish();
        }
        // Copy the goal-first keys in small chunks through a stack buffer.
        unsigned long long chunk[256];
        const unsigned long long* src = reinterpret_cast<const unsigned long long*>(b + kPathOff) + ctl.path_off;
        for (uint32_t at = 0; at < ctl.path_len; at += 256) {
            const uint32_t m = ctl.path_len - at < 256 ? ctl.path_len - at : 256;
            if ((e = cudaMemcpyAsync(chunk, src + at, m * 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
                (e = cudaStreamSynchronize(st)) != cudaSuccess)
                return fail(e, "path copy");
            out->d2h_bytes += m * 8;
            for (uint32_t j = 0; j < m; ++j)
                unpack_board(3, chunk[j], 0, path + (size_t)(ctl.path_len - 1 - (at + j)) * 9);
        }
    }
    return finish();
}
