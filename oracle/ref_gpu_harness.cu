// The reference's own GA* search, compiled unmodified for sm_103a.
//
// TEST INFRASTRUCTURE ONLY.  Built by `oracle/build.py --ref-gpu` from the
// reference headers staged (unmodified) in oracle/_ref/src, into
// oracle/_ref/libref_gpu.so; loaded by the GPU parity tests through ctypes.
// Nothing of the engine is linked in: the search below is the reference's
// a_star template (a_star.h:223-282) with its heaps, hashmaps, bitonic sorts
// and reductions, driven through its front ends SlidingPuzzle::solve<size>
// (a_star_sliding_puzzle.h:165-171) and Pathfinding::solve
// (a_star_pathfinding.h:223-238) on the reference's text input format.  The
// path is printed with the reference's own operator<< (one state per line,
// start first), as main.cu:26-29 prints it.
//
// Which inputs the reference handles is set by its code, not by this file:
// grid coordinates pass through 8 bits (a_star_pathfinding.h:185-186), so
// sides above 255 are out of its range; its sliding successor reaches only
// moves 0 and 2 (a_star_sliding_puzzle.h:106-111); num_queues must be a
// multiple of 16 (heaps.h:239-242).
#include <chrono>
#include <cstring>
#include <exception>
#include <sstream>
#include <string>

#include "a_star_sliding_puzzle.h"
#include "a_star_pathfinding.h"

namespace {

std::string g_error;

template <class R>
int emit(const R& r, char* out, size_t cap, double* search_ms) {
    std::ostringstream o;
    for (const auto& p : r.first) o << p << '\n';
    const std::string s = o.str();
    if (s.size() + 1 > cap) {
        g_error = "output buffer too small";
        return -3;
    }
    std::memcpy(out, s.c_str(), s.size() + 1);
    if (search_ms) *search_ms = std::chrono::duration<double, std::milli>(r.second).count();
    return (int)r.first.size();
}

}  // namespace

// kind 0: sliding puzzle of side n (3 or 4), text "start goal"
//         (a_star_sliding_puzzle.h:21-48, 167-168);
// kind 1: grid, text in the reference's pathfinding format
//         (a_star_pathfinding.h:83-128, 223-231).
// Returns the number of path states (0 = no path) or a negative error;
// `search_ms` gets the reference's own search-loop time (a_star.h:245, 266),
// `wall_ms` the whole solve including its allocations and path rebuild.
extern "C" int ref_gpu_solve(int kind, int n, const char* text, uint32_t num_queues, char* out,
                             size_t cap, double* search_ms, double* wall_ms) {
    try {
        std::istringstream in(text);
        in.exceptions(std::ios_base::failbit | std::ios_base::badbit);
        const auto t0 = std::chrono::steady_clock::now();
        int rc;
        if (kind == 1) {
            rc = emit(Pathfinding::solve(in, num_queues), out, cap, search_ms);
        } else if (n == 3) {
            rc = emit(SlidingPuzzle::solve<3>(in, num_queues), out, cap, search_ms);
        } else if (n == 4) {
            rc = emit(SlidingPuzzle::solve<4>(in, num_queues), out, cap, search_ms);
        } else {
            g_error = "only 3x3 and 4x4 boards are built";
            return -1;
        }
        cuda_check(cudaDeviceSynchronize());
        if (wall_ms)
            *wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        return rc;
    } catch (const std::exception& e) {
        g_error = e.what();
        return -2;
    }
}

extern "C" const char* ref_gpu_error() { return g_error.c_str(); }
