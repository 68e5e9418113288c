// The reference's own problem plugins on this engine's template API.
//
// TEST INFRASTRUCTURE ONLY.  The reference's front-end headers
// a_star_pathfinding.h and a_star_sliding_puzzle.h -- their Position types,
// successor functions, heuristics with their __constant__ data, text parsers
// and printers, and their solve() functions -- are compiled unmodified (from
// the copy staged in oracle/_ref/src) with include/gastar/a_star.cuh standing
// in for the reference's a_star.h: the include guard A_STAR_H keeps the
// reference's search out, so the a_star<T, max_neighbours, gen, h>(start,
// target, num_queues) call inside SlidingPuzzle::solve<size>
// (a_star_sliding_puzzle.h:165-171) and Pathfinding::solve
// (a_star_pathfinding.h:223-238) runs the engine's GA* kernel.  This is what
// a maintainer gets by swapping the header; nothing here restates a plugin.
#include <cstring>
#include <exception>
#include <sstream>
#include <string>

#include "gastar/a_star.cuh"

#define A_STAR_H
#include "a_star_pathfinding.h"
#include "a_star_sliding_puzzle.h"

namespace {

std::string g_error;

template <class R>
int emit(const R& r, char* out, size_t cap) {
    std::ostringstream o;
    for (const auto& p : r.first) o << p << '\n';
    const std::string s = o.str();
    if (s.size() + 1 > cap) {
        g_error = "output buffer too small";
        return -3;
    }
    std::memcpy(out, s.c_str(), s.size() + 1);
    return (int)r.first.size();
}

}  // namespace

// kind 0: sliding puzzle of side n (3, 4 or 5); kind 1: grid.  Text in the
// reference's input formats.  Returns the number of path states (0 = no
// path) or a negative error; the path goes to `out` in the reference's
// printed form.
extern "C" int refplug_solve(int kind, int n, const char* text, uint32_t num_queues, char* out,
                             size_t cap) {
    try {
        std::istringstream in(text);
        in.exceptions(std::ios_base::failbit | std::ios_base::badbit);
        if (kind == 1) return emit(Pathfinding::solve(in, num_queues), out, cap);
        if (n == 3) return emit(SlidingPuzzle::solve<3>(in, num_queues), out, cap);
        if (n == 4) return emit(SlidingPuzzle::solve<4>(in, num_queues), out, cap);
        if (n == 5) return emit(SlidingPuzzle::solve<5>(in, num_queues), out, cap);
        g_error = "board side must be 3, 4 or 5";
        return -1;
    } catch (const std::exception& e) {
        g_error = e.what();
        return -2;
    }
}

extern "C" const char* refplug_error() { return g_error.c_str(); }
