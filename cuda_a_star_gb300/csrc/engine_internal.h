// Internal host-side declarations shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/gastar.h"
#include "engine_types.h"

namespace gastar {

struct DevBuf {
    void* p = nullptr;
    size_t n = 0;
    bool fresh = false;         // set when ensure() reallocated (contents undefined)
    bool ensure(size_t bytes);  // grows (contents are not kept)
    void release();
};

void set_error(const std::string& s);
bool cuda_ok(cudaError_t e, const char* what);

const void* search_kernel_for(uint32_t kinds, uint32_t threads);
uint32_t entry_bytes(uint32_t kind);
uint32_t max_neighbours(uint32_t kind);
uint32_t key_words(uint32_t kind);
size_t block_smem_bytes(uint32_t kinds, uint32_t warps, uint32_t ew, bool multi,
                        uint32_t heap_snodes = kHeapSmemNodes, bool buckets = false);
int launch_search(struct ::gastar_ctx* c, uint32_t kinds, const LaunchParams& P, uint32_t blocks,
                  uint32_t threads, size_t smem, cudaStream_t st);
// Rebuilds the paths of finished instances into `arena` (see path_kernel):
// with `offs` (device, n + 1 prefix offsets) each instance writes its own
// slice in one walk.
int launch_paths(const InstDesc* d_insts, uint32_t n, unsigned long long* arena,
                 unsigned long long arena_words, unsigned long long* used, cudaStream_t st,
                 const unsigned long long* offs = nullptr);
// Largest count of shared-memory heap nodes per warp (>= kHeapSmemNodes) that
// keeps `blocks_per_sm` blocks of this shape resident; *smem = the block's
// dynamic shared memory with it.
uint32_t fit_heap_snodes(gastar_ctx* c, uint32_t kinds, uint32_t warps, uint32_t ew, bool multi, uint32_t threads,
                         int blocks_per_sm, size_t* smem, bool buckets = false);
int occupancy_blocks(struct ::gastar_ctx* c, uint32_t kinds, uint32_t threads, size_t smem);
int device_min_weight(struct ::gastar_ctx* c, const uint8_t* d_w, uint64_t cells, cudaStream_t st,
                      uint32_t* out);
// Places a grid's weights from the caller's host buffer at d_dst and returns
// its least passable weight (255: none); synchronises `st`, so the caller may
// reuse the buffer afterwards.  By the context's upload_mode: staged (host
// threads and a pinned ring), read in place by one kernel that also reduces
// (where the GPU reads pageable host memory through the host's page tables),
// or a copy, then device_min_weight.
int upload_grid(struct ::gastar_ctx* c, uint8_t* d_dst, const uint8_t* h_src, uint64_t cells, cudaStream_t st,
                uint32_t* minw);
// The staged way (upload.cpp): host threads fill pinned chunks and reduce the
// least weight while the previous chunks are sent.
struct HostStager;
int upload_grid_staged(struct ::gastar_ctx* c, uint8_t* d_dst, const uint8_t* h_src, uint64_t cells,
                       cudaStream_t st, uint32_t* minw);
void destroy_stager(HostStager* s);

struct PlainProblem {
    uint32_t kind, n;
    uint64_t start0, start1, goal0, goal1;
    const uint8_t* d_weights;  // grid (device)
    uint32_t W, H, minw, f0;
};
// One instance on a multi-block team (the plain engine); path_keys receives
// the path goal-first (KW words per state) when not null.
int plain_solve(struct ::gastar_ctx* c, const PlainProblem& pp, const gastar_config* user_cfg,
                std::vector<uint64_t>* path_keys, gastar_result* out);

bool valid_board(uint32_t n, const uint8_t* b);
void pack_board(uint32_t n, const uint8_t* b, uint64_t& lo, uint64_t& hi);
void unpack_board(uint32_t n, uint64_t lo, uint64_t hi, uint8_t* b);
uint32_t sliding_h(uint32_t n, const uint8_t* b, const uint8_t* goal, uint32_t heuristic);
bool sliding_solvable(uint32_t n, const uint8_t* s, const uint8_t* g);
uint32_t grid_h(uint32_t x, uint32_t y, uint32_t tx, uint32_t ty, uint32_t minw, uint32_t heuristic);
uint64_t next_pow2(uint64_t v);
// Least non-zero weight of a grid, 255 if none (vectorised scan).
uint8_t min_passable_weight(const uint8_t* weights, size_t cells);

}  // namespace gastar

struct gastar_ctx {
    int device = 0;
    int sms = 0;
    int coop = 0;
    size_t smem_per_sm = 0;  // shared memory of one SM
    size_t smem_optin = 0;   // largest dynamic shared memory one block may ask for
    size_t mem_total = 0;
    char name[256] = {0};
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    gastar::DevBuf table, dense, touched, heaps, hdr, stage, path, misc, weights, buckets;
    // Plain engine: descriptor, control block, team control and counters of
    // one solve in one device block, uploaded from a pinned mirror in one copy.
    gastar::DevBuf launch;
    void* h_launch = nullptr;      // pinned
    uint64_t* h_path = nullptr;    // pinned: the path's first words, read back with the control block
    bool can_read_host = false;    // kernels read pageable host memory through the host's
                                   // page tables (ATS over NVLink-C2C on Grace)
    int upload_mode = 2;           // grid uploads: 0 copy, 1 read in place, 2 staged
    gastar::HostStager* stager = nullptr;  // staged uploads (pinned ring, host threads)
    bool table_dirty = true;       // hash table needs a full clear before the next solve
    uint32_t prev_slot_words = 2;  // slot width of the solve that filled the touched list
    uint64_t launches = 0;         // kernels launched by this context
    gastar::InstCtl* h_ctl = nullptr;  // pinned
};
