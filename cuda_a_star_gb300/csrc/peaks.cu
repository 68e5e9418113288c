// Random-access peaks of the device, the roofline denominators of the hash
// and heap kernels: the search touches its duplicate-detection table in
// random 16-byte slots and its heaps in random 512-byte nodes, so its bound is
// the rate of independent random 32-byte sector accesses, not the streaming
// copy bandwidth.  Two kernels measure it over a buffer far larger than L2:
//   * gather: random 32-byte loads (one sector each), L2 bypassed for reuse;
//   * cas:    random 16-byte compare-and-swaps (atom.cas.b128), the table's
//             claim operation, on a buffer of empty slots.
// Every thread keeps kInFlight independent accesses outstanding; the grid
// fills every SM.  Result = sectors x 32 bytes / kernel time.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/gastar.h"
#include "device_common.cuh"
#include "engine_internal.h"

namespace {

using namespace gastar;

constexpr int kInFlight = 8;

__global__ void __launch_bounds__(256) gather_kernel(const ulonglong2* buf, uint64_t sectors_mask,
                                                     uint32_t rounds, uint64_t seed,
                                                     unsigned long long* sink) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t x = mix64(seed ^ (tid * 0x9e3779b97f4a7c15ull));
    unsigned long long acc = 0;
    for (uint32_t r = 0; r < rounds; ++r) {
        ulonglong2 v[kInFlight][2];
#pragma unroll
        for (int j = 0; j < kInFlight; ++j) {
            x = mix64(x + (uint64_t)j + 1);
            const uint64_t s = x & sectors_mask;  // one 32-byte sector
            v[j][0] = __ldcg(buf + 2 * s);
            v[j][1] = __ldcg(buf + 2 * s + 1);
        }
#pragma unroll
        for (int j = 0; j < kInFlight; ++j) acc += v[j][0].x ^ v[j][1].y;
    }
    if (acc == 0x5a5a5a5a5a5a5a5aull) *sink = acc;  // keeps the loads
}

__global__ void __launch_bounds__(256) cas_kernel(unsigned long long* buf, uint64_t slots_mask,
                                                  uint32_t rounds, uint64_t seed,
                                                  unsigned long long* sink) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t x = mix64(seed ^ (tid * 0x9e3779b97f4a7c15ull));
    unsigned long long acc = 0;
    for (uint32_t r = 0; r < rounds; ++r) {
        uint64_t o0[kInFlight], o1[kInFlight];
#pragma unroll
        for (int j = 0; j < kInFlight; ++j) {
            x = mix64(x + (uint64_t)j + 1);
            const uint64_t s = x & slots_mask;  // one 16-byte slot
            cas128(buf + 2 * s, kEmpty, kEmpty, x, tid, o0[j], o1[j]);
        }
#pragma unroll
        for (int j = 0; j < kInFlight; ++j) acc += o0[j] ^ o1[j];
    }
    if (acc == 0x5a5a5a5a5a5a5a5aull) *sink = acc;
}

}  // namespace

extern "C" int gastar_measure_random_peak(gastar_ctx* ctx, uint64_t buffer_bytes, uint32_t kind,
                                          double* gbs, double* ms) {
    if (!ctx || !gbs || kind > 1) return GASTAR_BAD_INPUT;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return GASTAR_CUDA_ERROR;
    uint64_t bytes = 1ull << 30;
    while (bytes * 2 <= buffer_bytes) bytes *= 2;  // a power of two, >= 1 GiB
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
    const uint32_t rounds = 64;
    const double accesses = (double)blocks * threads * rounds * kInFlight;
    float t = 0;
    for (int rep = 0; rep < 3 && rc == GASTAR_OK; ++rep) {  // the first run warms up
        cudaEventRecord(ctx->e0, st);
        if (kind == 0)
            gather_kernel<<<blocks, threads, 0, st>>>(static_cast<const ulonglong2*>(buf), bytes / 32 - 1,
                                                      rounds, 0x1234 + rep, sink);
        else
            cas_kernel<<<blocks, threads, 0, st>>>(static_cast<unsigned long long*>(buf), bytes / 16 - 1,
                                                   rounds, 0x1234 + rep, sink);
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
