// Random-access peaks of the device, the roofline denominators of the hash
// and heap kernels: the search touches its duplicate-detection table in
// random 16-byte slots and its heaps in random 512-byte nodes, so its bound is
// the rate of independent random 32-byte sector accesses, not the streaming
// copy bandwidth.  Two kernels measure it over a buffer far larger than L2:
//   * gather: random 32-byte loads (one sector each), L2 bypassed for reuse;
//   * cas:    random 16-byte compare-and-swaps (atom.cas.b128), the table's
//             claim operation, on a buffer of empty slots.
// Every thread keeps a fixed number of independent accesses outstanding (8
// by default; the sweep entry point varies it, the buffer size and the loads
// per sector); the grid fills every SM.  Result = sectors x 32 bytes / kernel
// time.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "../../include/gastar.h"
#include "device_common.cuh"
#include "engine_internal.h"

namespace {

using namespace gastar;

// IF independent accesses in flight per thread; HALVES = 16-byte loads per
// 32-byte sector (1 or 2: either moves the whole sector from DRAM).
template <int IF, int HALVES>
__global__ void __launch_bounds__(256) gather_kernel(const ulonglong2* buf, uint64_t sectors_mask,
                                                     uint32_t rounds, uint64_t seed,
                                                     unsigned long long* sink) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t x = mix64(seed ^ (tid * 0x9e3779b97f4a7c15ull));
    unsigned long long acc = 0;
    for (uint32_t r = 0; r < rounds; ++r) {
        ulonglong2 v[IF][HALVES];
#pragma unroll
        for (int j = 0; j < IF; ++j) {
            x = mix64(x + (uint64_t)j + 1);
            const uint64_t s = x & sectors_mask;  // one 32-byte sector
#pragma unroll
            for (int k = 0; k < HALVES; ++k) v[j][k] = __ldcg(buf + 2 * s + k);
        }
#pragma unroll
        for (int j = 0; j < IF; ++j) acc += v[j][0].x ^ v[j][HALVES - 1].y;
    }
    if (acc == 0x5a5a5a5a5a5a5a5aull) *sink = acc;  // keeps the loads
}

template <int IF>
__global__ void __launch_bounds__(256) cas_kernel(unsigned long long* buf, uint64_t slots_mask,
                                                  uint32_t rounds, uint64_t seed,
                                                  unsigned long long* sink) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t x = mix64(seed ^ (tid * 0x9e3779b97f4a7c15ull));
    unsigned long long acc = 0;
    for (uint32_t r = 0; r < rounds; ++r) {
        uint64_t o0[IF], o1[IF];
#pragma unroll
        for (int j = 0; j < IF; ++j) {
            x = mix64(x + (uint64_t)j + 1);
            const uint64_t s = x & slots_mask;  // one 16-byte slot
            cas128(buf + 2 * s, kEmpty, kEmpty, x, tid, o0[j], o1[j]);
        }
#pragma unroll
        for (int j = 0; j < IF; ++j) acc += o0[j] ^ o1[j];
    }
    if (acc == 0x5a5a5a5a5a5a5a5aull) *sink = acc;
}

template <int IF>
void launch_one(uint32_t kind, uint32_t halves, uint32_t blocks, uint32_t threads, void* buf, uint64_t bytes,
                uint32_t rounds, uint64_t seed, unsigned long long* sink, cudaStream_t st) {
    if (kind == 1)
        cas_kernel<IF><<<blocks, threads, 0, st>>>(static_cast<unsigned long long*>(buf), bytes / 16 - 1,
                                                   rounds, seed, sink);
    else if (halves == 1)
        gather_kernel<IF, 1><<<blocks, threads, 0, st>>>(static_cast<const ulonglong2*>(buf), bytes / 32 - 1,
                                                         rounds, seed, sink);
    else
        gather_kernel<IF, 2><<<blocks, threads, 0, st>>>(static_cast<const ulonglong2*>(buf), bytes / 32 - 1,
                                                         rounds, seed, sink);
}

int measure(gastar_ctx* ctx, uint64_t bytes, uint32_t kind, uint32_t in_flight, uint32_t halves, double* gbs,
            double* ms) {
    if (cudaSetDevice(ctx->device) != cudaSuccess) return GASTAR_CUDA_ERROR;
    void* buf = nullptr;
    unsigned long long* sink = nullptr;
    if (cudaMalloc(&buf, bytes) != cudaSuccess) return GASTAR_OUT_OF_MEMORY;
    if (cudaMalloc(&sink, 8) != cudaSuccess) {
        cudaFree(buf);
        return GASTAR_OUT_OF_MEMORY;
    }
    cudaStream_t st = ctx->stream;
    int rc = GASTAR_OK;
    cudaMemsetAsync(buf, 0xff, bytes, st);  // empty slots for the CAS kernel
    const uint32_t threads = 256, blocks = (uint32_t)ctx->sms * 8;
    // About 64 x 8 accesses per thread whatever the depth in flight.
    const uint32_t rounds = std::max(8u, 512u / in_flight);
    const double accesses = (double)blocks * threads * rounds * in_flight;
    float t = 0;
    for (int rep = 0; rep < 3 && rc == GASTAR_OK; ++rep) {  // the first run warms up
        cudaEventRecord(ctx->e0, st);
        switch (in_flight) {
            case 1: launch_one<1>(kind, halves, blocks, threads, buf, bytes, rounds, 0x1234 + rep, sink, st); break;
            case 2: launch_one<2>(kind, halves, blocks, threads, buf, bytes, rounds, 0x1234 + rep, sink, st); break;
            case 4: launch_one<4>(kind, halves, blocks, threads, buf, bytes, rounds, 0x1234 + rep, sink, st); break;
            case 16: launch_one<16>(kind, halves, blocks, threads, buf, bytes, rounds, 0x1234 + rep, sink, st); break;
            case 32: launch_one<32>(kind, halves, blocks, threads, buf, bytes, rounds, 0x1234 + rep, sink, st); break;
            default: launch_one<8>(kind, halves, blocks, threads, buf, bytes, rounds, 0x1234 + rep, sink, st); break;
        }
        cudaEventRecord(ctx->e1, st);
        if (cudaEventSynchronize(ctx->e1) != cudaSuccess || cudaGetLastError() != cudaSuccess)
            rc = GASTAR_CUDA_ERROR;
        else
            cudaEventElapsedTime(&t, ctx->e0, ctx->e1);
    }
    cudaFree(sink);
    cudaFree(buf);
    if (rc != GASTAR_OK) return rc;
    *gbs = accesses * 32.0 / ((double)t * 1e-3) / 1e9;
    if (ms) *ms = t;
    return GASTAR_OK;
}

}  // namespace

extern "C" int gastar_measure_random_peak(gastar_ctx* ctx, uint64_t buffer_bytes, uint32_t kind,
                                          double* gbs, double* ms) {
    if (!ctx || !gbs || kind > 1) return GASTAR_BAD_INPUT;
    uint64_t bytes = 1ull << 30;
    while (bytes * 2 <= buffer_bytes) bytes *= 2;  // a power of two, >= 1 GiB
    return measure(ctx, bytes, kind, 8, 2, gbs, ms);
}

extern "C" int gastar_measure_random_peak_ex(gastar_ctx* ctx, uint64_t buffer_bytes, uint32_t kind,
                                             uint32_t in_flight, uint32_t loads_per_sector, double* gbs,
                                             double* ms) {
    if (!ctx || !gbs || kind > 1 || buffer_bytes < (1ull << 20)) return GASTAR_BAD_INPUT;
    if (in_flight != 1 && in_flight != 2 && in_flight != 4 && in_flight != 8 && in_flight != 16 &&
        in_flight != 32)
        return GASTAR_BAD_INPUT;
    if (loads_per_sector != 1 && loads_per_sector != 2) return GASTAR_BAD_INPUT;
    uint64_t bytes = 1ull << 20;
    while (bytes * 2 <= buffer_bytes) bytes *= 2;  // a power of two, >= 1 MiB
    return measure(ctx, bytes, kind, in_flight, loads_per_sector, gbs, ms);
}
