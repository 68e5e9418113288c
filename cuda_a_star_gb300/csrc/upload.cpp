// Grid uploads from the caller's pageable host buffer.
//
// Three ways, chosen per context at gastar_create (GASTAR_UPLOAD):
//  * staged (default): host threads copy the buffer into a ring of pinned
//    chunks and reduce its least passable weight while they copy; each filled
//    chunk goes to the device by DMA while the next one is copied.  The
//    threads walk the caller's pages with the CPU's own page tables, so the
//    rate holds on pages the GPU has never seen (measured 57-59 GB/s on 3 GB
//    of freshly generated grids on a GB300 host, where in-place reads ran at
//    4-5 GB/s and the driver's pageable copy at 3-4 GB/s; on other hosts
//    those two ranged 7-37 and 3-15 GB/s);
//  * in place: one kernel reads the buffer through the host's page tables
//    (Grace: NVLink-C2C) and reduces in the same pass (copy_min_kernel);
//  * copy: cudaMemcpyAsync from the pageable buffer, then min_weight_kernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/gastar.h"
#include "engine_internal.h"

namespace gastar {

namespace {

// A few persistent threads that run the parts of one job together with the
// calling thread (parts are claimed from an atomic counter).
class CopyPool {
   public:
    explicit CopyPool(int workers) {
        for (int i = 0; i < workers; ++i) th_.emplace_back([this] { work(); });
    }
    ~CopyPool() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto& t : th_) t.join();
    }
    int threads() const { return (int)th_.size() + 1; }
    // Runs fn(0) .. fn(parts - 1); returns when every part has finished.
    void run(int parts, const std::function<void(int)>& fn) {
        {
            std::lock_guard<std::mutex> lk(mu_);
            fn_ = &fn;
            parts_ = parts;
            next_.store(0);
            ++gen_;
        }
        cv_.notify_all();
        for (int p; (p = next_.fetch_add(1)) < parts;) fn(p);
        std::unique_lock<std::mutex> lk(mu_);
        done_.wait(lk, [&] { return active_ == 0; });
        fn_ = nullptr;
    }

   private:
    void work() {
        uint64_t seen = 0;
        std::unique_lock<std::mutex> lk(mu_);
        for (;;) {
            cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
            if (stop_) return;
            seen = gen_;
            if (!fn_) continue;  // the job finished before this thread woke
            const std::function<void(int)>* fn = fn_;
            const int parts = parts_;
            ++active_;
            lk.unlock();
            for (int p; (p = next_.fetch_add(1)) < parts;) (*fn)(p);
            lk.lock();
            if (--active_ == 0) done_.notify_all();
        }
    }
    std::vector<std::thread> th_;
    std::mutex mu_;
    std::condition_variable cv_, done_;
    const std::function<void(int)>* fn_ = nullptr;
    int parts_ = 0, active_ = 0;
    std::atomic<int> next_{0};
    uint64_t gen_ = 0;
    bool stop_ = false;
};

// Copies n bytes and returns min(w - 1) over them, 0 wrapping to 255 (a
// loop the compiler vectorises).
uint8_t copy_min_bytes(unsigned char* dst, const unsigned char* src, size_t n) {
    uint8_t m = 255;
    for (size_t i = 0; i < n; ++i) {
        const uint8_t t = src[i];
        dst[i] = t;
        const uint8_t u = (uint8_t)(t - 1u);
        m = u < m ? u : m;
    }
    return m;
}

}  // namespace

struct HostStager {
    static constexpr size_t kChunk = 8ull << 20;  // bytes per pinned chunk
    static constexpr int kSlots = 4;              // chunks in flight
    unsigned char* pinned = nullptr;
    cudaEvent_t ev[kSlots] = {};
    CopyPool pool;
    explicit HostStager(int workers) : pool(workers) {}
    ~HostStager() {
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        if (pinned) cudaFreeHost(pinned);
    }
};

void destroy_stager(HostStager* s) { delete s; }

namespace {

// Nothing may throw across the C ABI: a stager that cannot start its threads
// or allocate reports failure, and the upload falls back to a copy.
HostStager* stager(gastar_ctx* c) {
    if (c->stager) return c->stager;
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    HostStager* s = nullptr;
    try {
        s = new HostStager((int)std::min(8u, std::max(1u, hw / 2)) - 1);
    } catch (...) {
        set_error("grid upload: could not start the staging threads");
        return nullptr;
    }
    bool ok = cuda_ok(cudaMallocHost(reinterpret_cast<void**>(&s->pinned), HostStager::kChunk * HostStager::kSlots),
                      "cudaMallocHost");
    for (auto& e : s->ev) ok = ok && cuda_ok(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
    if (!ok) {
        delete s;
        return nullptr;
    }
    c->stager = s;
    return s;
}

}  // namespace

int upload_grid_staged(gastar_ctx* c, uint8_t* d_dst, const uint8_t* h_src, uint64_t cells, cudaStream_t st,
                       uint32_t* minw) {
    HostStager* hs = stager(c);
    if (!hs) return GASTAR_OUT_OF_MEMORY;
    const int threads = hs->pool.threads();
    std::vector<uint8_t> part_min((size_t)threads, 255);
    uint8_t m = 255;
    uint64_t k = 0;
    for (uint64_t off = 0; off < cells; off += HostStager::kChunk, ++k) {
        const size_t n = (size_t)std::min<uint64_t>(HostStager::kChunk, cells - off);
        const int slot = (int)(k % HostStager::kSlots);
        // The chunk's previous contents have reached the device.
        if (k >= (uint64_t)HostStager::kSlots && !cuda_ok(cudaEventSynchronize(hs->ev[slot]), "cudaEventSynchronize"))
            return GASTAR_CUDA_ERROR;
        unsigned char* buf = hs->pinned + (size_t)slot * HostStager::kChunk;
        const int parts = n >= (1u << 20) ? threads : 1;
        const size_t per = (n + parts - 1) / parts;
        const uint8_t* src = h_src + off;
        try {
            hs->pool.run(parts, [&](int p) {
                const size_t lo = (size_t)p * per, hi = std::min(n, lo + per);
                part_min[p] = lo < hi ? copy_min_bytes(buf + lo, src + lo, hi - lo) : 255;
            });
        } catch (...) {  // std::function or locking failed: nothing was sent from this chunk
            if (!cuda_ok(cudaStreamSynchronize(st), "cudaStreamSynchronize")) return GASTAR_CUDA_ERROR;
            set_error("grid upload: staging failed");
            return GASTAR_CUDA_ERROR;
        }
        for (int p = 0; p < parts; ++p) m = std::min(m, part_min[p]);
        if (!cuda_ok(cudaMemcpyAsync(d_dst + off, buf, n, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync") ||
            !cuda_ok(cudaEventRecord(hs->ev[slot], st), "cudaEventRecord"))
            return GASTAR_CUDA_ERROR;
    }
    if (!cuda_ok(cudaStreamSynchronize(st), "cudaStreamSynchronize")) return GASTAR_CUDA_ERROR;
    *minw = m == 255 ? 255u : m + 1u;
    return GASTAR_OK;
}

}  // namespace gastar
