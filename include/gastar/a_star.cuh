// Header-only generic GA* with the reference's template API.
//
//   template <typename T, unsigned char max_neighbours,
//             NeighbourGenerator<T> neighbour_generator, Heuristic<T> heuristic,
//             uint16_t bucket_depth = 256>
//   std::pair<std::vector<T>, std::chrono::nanoseconds>
//   a_star(const T& start, const T& target, uint32_t num_queues);
//
// Same signature, plugin types and result as the reference (a_star.h:223-224,
// functional_types.h:6-10): the path from start to target (empty when the
// target is unreachable) and the search time.  Compile the including file
// with nvcc for sm_103a.  Requirements on T: trivially copyable, at most 32
// bytes, equal states have equal bytes (deterministic padding).  The search
// runs on the engine's warp-heap GA* kernel (plugin domain: full heuristic
// call per successor, parents recorded by table slot).  `bucket_depth` only
// keeps the signature; the table is open addressing.  CUDA errors throw
// std::runtime_error like the reference's cuda_check (helpers.h:46-50).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../cuda_a_star_gb300/csrc/plugin.cuh"

template <typename T>
using NeighbourGenerator = void (*)(const T& source, T& target, bool& target_exists, uint32_t& cost,
                                    unsigned char i);
template <typename T>
using Heuristic = uint32_t (*)(const T&);

namespace gastar {
namespace plugin_host {

inline void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorName(e));
}

struct Buffer {
    void* p = nullptr;
    size_t n = 0;
    void ensure(size_t bytes) {
        if (bytes <= n) return;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        check(cudaMalloc(&p, bytes), "cudaMalloc");
        n = bytes;
    }
    ~Buffer() {
        if (p) cudaFree(p);
    }
};

// Search parameters of the template API (defaults of the C ABI's plain engine).
struct Options {
    uint32_t expansion_width = 32;
    uint32_t warps_per_block = 4;
    uint32_t table_log2 = 20;      // first table size; grows x4 on overflow
    uint32_t max_table_log2 = 28;
    float load_factor = 0.75f;
};

template <class D, typename T>
std::pair<std::vector<T>, std::chrono::nanoseconds> solve(const T& start, const T& target, uint32_t num_queues,
                                                          const Options& o = Options()) {
    constexpr int KW = D::KW;
    using E = Entry<KW>;
    int dev = 0;
    check(cudaGetDevice(&dev), "cudaGetDevice");
    cudaDeviceProp prop;
    check(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties");
    const uint32_t ew = std::min(32u, std::max(1u, o.expansion_width));
    const uint32_t W = std::min(8u, std::max(1u, o.warps_per_block));
    const uint32_t threads = W * 32;
    const uint64_t Q = num_queues ? num_queues : 4096;
    uint64_t heaps = (Q + ew - 1) / ew, blocks = (heaps + W - 1) / W;
    const bool multi = blocks > 1;
    const size_t smem = (multi ? 0 : 2 * stage_entries_per_buffer(W, ew, D::MAXN) * sizeof(E)) +
                        (size_t)W * (kHeapSmemNodes - 1) * 32 * sizeof(E);
    const void* kern = reinterpret_cast<const void*>(&plugin_search_kernel<D>);
    if (smem > kSmemNoOptIn)
        check(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
              "cudaFuncSetAttribute");
    int nb = 0;
    check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, (int)threads, smem), "occupancy");
    blocks = std::min<uint64_t>(blocks, (uint64_t)nb * prop.multiProcessorCount);
    if (blocks == 0) throw std::runtime_error("gastar: kernel does not fit on the device");
    heaps = blocks * W;

    uint64_t key_lo[2] = {0, 0}, key_hi[2] = {0, 0}, goal_lo[2] = {0, 0}, goal_hi[2] = {0, 0};
    {
        uint64_t w[4] = {0, 0, 0, 0}, v[4] = {0, 0, 0, 0};
        std::memcpy(w, &start, sizeof(T));
        std::memcpy(v, &target, sizeof(T));
        key_lo[0] = w[0], key_lo[1] = w[1], key_hi[0] = w[2], key_hi[1] = w[3];
        goal_lo[0] = v[0], goal_lo[1] = v[1], goal_hi[0] = v[2], goal_hi[1] = v[3];
    }
    Buffer table, heapmem, hdr, stage, desc, ctl, team, path, used;
    cudaEvent_t e0, e1;
    check(cudaEventCreate(&e0), "cudaEventCreate");
    check(cudaEventCreate(&e1), "cudaEventCreate");
    std::chrono::nanoseconds elapsed(0);
    std::vector<T> result;
    uint32_t log2 = o.table_log2;
    for (;;) {
        const uint64_t slots = 1ull << log2;
        const uint64_t words = slots * D::Tab::SW;
        const uint64_t entries = slots;
        const uint64_t cap = std::max<uint64_t>(2 * kHeapSmemNodes, (2 * entries / heaps + 31) / 32);
        table.ensure(words * 8);
        heapmem.ensure(heaps * (cap + 1) * 32 * sizeof(E));
        hdr.ensure(heaps * 8);
        stage.ensure(multi ? team_stage_bytes((uint32_t)blocks, W, ew, D::MAXN, sizeof(E)) : 16);
        desc.ensure(sizeof(InstDesc));
        ctl.ensure(sizeof(InstCtl));
        team.ensure(sizeof(TeamCtl) + 64);
        InstDesc d;
        std::memset(&d, 0, sizeof(d));
        d.kind = KIND_PLUGIN;
        d.start0 = key_lo[0], d.start1 = key_lo[1], d.start_hi[0] = key_hi[0], d.start_hi[1] = key_hi[1];
        d.goal0 = goal_lo[0], d.goal1 = goal_lo[1], d.goal_hi[0] = goal_hi[0], d.goal_hi[1] = goal_hi[1];
        d.table = static_cast<unsigned long long*>(table.p);
        d.table_words = words;
        d.table_mask = slots - 1;
        d.table_limit = (uint64_t)((double)slots * o.load_factor);
        d.max_probe = 4096;
        d.heaps = (uint32_t)heaps;
        d.heap_nodes = heapmem.p;
        d.heap_hdr = static_cast<uint32_t*>(hdr.p);
        d.heap_cap = (uint32_t)cap;
        d.ew = ew;
        d.ctl = static_cast<InstCtl*>(ctl.p);
        TeamCtl tc;
        team_ctl_init(tc);
        check(cudaMemcpy(desc.p, &d, sizeof(d), cudaMemcpyHostToDevice), "cudaMemcpy");
        check(cudaMemset(ctl.p, 0, sizeof(InstCtl)), "cudaMemset");
        check(cudaMemcpy(team.p, &tc, sizeof(tc), cudaMemcpyHostToDevice), "cudaMemcpy");
        check(cudaMemset(static_cast<char*>(team.p) + sizeof(TeamCtl), 0, 16), "cudaMemset");
        LaunchParams P;
        std::memset(&P, 0, sizeof(P));
        P.insts = static_cast<const InstDesc*>(desc.p);
        P.n_insts = 1;
        P.next = reinterpret_cast<uint32_t*>(static_cast<char*>(team.p) + sizeof(TeamCtl));
        P.team_ctas = (uint32_t)blocks;
        P.team = static_cast<TeamCtl*>(team.p);
        P.stage = stage.p;
        P.barrier_timeout_ns = 2000000000ull;
        void* args[] = {&P};
        check(cudaEventRecord(e0), "cudaEventRecord");
        if (multi)
            check(cudaLaunchCooperativeKernel(kern, dim3((unsigned)blocks), dim3(threads), args, smem, 0),
                  "cudaLaunchCooperativeKernel");
        else
            check(cudaLaunchKernel(kern, dim3(1), dim3(threads), args, smem, 0), "cudaLaunchKernel");
        check(cudaEventRecord(e1), "cudaEventRecord");
        InstCtl c;
        check(cudaMemcpy(&c, ctl.p, sizeof(c), cudaMemcpyDeviceToHost), "cudaMemcpy");
        float ms = 0;
        check(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
        elapsed += std::chrono::nanoseconds((long long)((double)ms * 1e6));
        if ((c.status == ST_TABLE_FULL || c.status == ST_HEAP_FULL) && log2 + 2 <= o.max_table_log2) {
            log2 += 2;
            continue;
        }
        if (c.status == ST_OK) {
            const uint64_t pw = ((uint64_t)c.best + 2) * KW;
            path.ensure(pw * 8);
            used.ensure(16);
            check(cudaMemset(used.p, 0, 8), "cudaMemset");
            plugin_path_kernel<D><<<1, 32>>>(P.insts, static_cast<unsigned long long*>(path.p), pw,
                                             static_cast<unsigned long long*>(used.p));
            check(cudaGetLastError(), "plugin_path_kernel");
            check(cudaMemcpy(&c, ctl.p, sizeof(c), cudaMemcpyDeviceToHost), "cudaMemcpy");
            if (c.status == ST_OK) {
                std::vector<unsigned long long> keys((size_t)c.path_len * KW);
                check(cudaMemcpy(keys.data(), static_cast<unsigned long long*>(path.p) + c.path_off,
                                 keys.size() * 8, cudaMemcpyDeviceToHost), "cudaMemcpy");
                for (uint32_t i = c.path_len; i-- > 0;) {  // stored goal-first
                    alignas(T) unsigned char buf[sizeof(T)];
                    std::memcpy(buf, keys.data() + (size_t)i * KW, sizeof(T));
                    result.push_back(*reinterpret_cast<const T*>(buf));
                }
            }
        } else if (c.status != ST_NO_PATH) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            throw std::runtime_error("gastar: search ended with status " + std::to_string(c.status));
        }
        break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return {std::move(result), elapsed};
}

}  // namespace plugin_host
}  // namespace gastar

template <typename T, unsigned char max_neighbours, NeighbourGenerator<T> neighbour_generator,
          Heuristic<T> heuristic, uint16_t bucket_depth = 256>
std::pair<std::vector<T>, std::chrono::nanoseconds> a_star(const T& start, const T& target,
                                                           const uint32_t num_queues) {
    using D = gastar::PluginDom<T, max_neighbours, neighbour_generator, heuristic>;
    return gastar::plugin_host::solve<D, T>(start, target, num_queues);
}
