// Test harness for the generic template API (include/gastar/a_star.cuh) and
// the reference-compatible front ends (include/gastar/reference_api.cuh).
// TEST INFRASTRUCTURE ONLY: built into a shared library by the GPU tests and
// called through ctypes.  Every entry returns the path length (states) or a
// negative value on error; paths are written start first.
#include <cstdint>
#include <cstring>
#include <vector>

#include "gastar/reference_api.cuh"

namespace {

// A plugin with no counterpart in the reference: the number line, where a
// state can step +1 or -1 (cost 1) or double (cost 3) within [0, limit).
struct Line {
    uint32_t v;
};
__constant__ uint32_t line_limit;
__constant__ uint32_t line_target;

__device__ void line_gen(const Line& s, Line& t, bool& ex, uint32_t& cost, unsigned char i) {
    ex = false;
    if (i == 0 && s.v + 1 < line_limit) { t.v = s.v + 1; cost = 1; ex = true; }
    if (i == 1 && s.v > 0) { t.v = s.v - 1; cost = 1; ex = true; }
    if (i == 2 && s.v * 2 < line_limit) { t.v = s.v * 2; cost = 3; ex = true; }
}
__device__ uint32_t line_h(const Line&) { return 0; }

template <unsigned char N>
int sliding(const uint8_t* start, const uint8_t* goal, uint32_t q, int ref_h, uint8_t* out) {
    SlidingPuzzle::Position<N> s(start), g(goal);
    SlidingPuzzle::set_manhattan_heuristic_target(g);
    std::pair<std::vector<SlidingPuzzle::Position<N>>, std::chrono::nanoseconds> r =
        ref_h ? a_star<SlidingPuzzle::Position<N>, 4, SlidingPuzzle::neighbour_generator<N>,
                       SlidingPuzzle::manhattan_heuristic<N>>(s, g, q)
              : a_star<SlidingPuzzle::Position<N>, 4, SlidingPuzzle::neighbour_generator<N>,
                       SlidingPuzzle::admissible_manhattan_heuristic<N>>(s, g, q);
    for (size_t i = 0; i < r.first.size(); ++i)
        for (int a = 0; a < N; ++a)
            for (int b = 0; b < N; ++b) out[i * N * N + a * N + b] = r.first[i].board[a][b];
    return (int)r.first.size();
}

}  // namespace

extern "C" int harness_sliding(uint32_t n, const uint8_t* start, const uint8_t* goal, uint32_t q, int ref_h,
                               uint8_t* out) {
    try {
        if (n == 3) return sliding<3>(start, goal, q, ref_h, out);
        if (n == 4) return sliding<4>(start, goal, q, ref_h, out);
        if (n == 5) return sliding<5>(start, goal, q, ref_h, out);
    } catch (...) {
        return -2;
    }
    return -1;
}

extern "C" int harness_grid(uint32_t w, uint32_t h, const uint8_t* weights, uint32_t sx, uint32_t sy,
                            uint32_t tx, uint32_t ty, uint32_t q, uint32_t* out) {
    try {
        uint8_t* d = nullptr;
        gastar::plugin_host::check(cudaMalloc(&d, (size_t)w * h), "cudaMalloc");
        gastar::plugin_host::check(cudaMemcpy(d, weights, (size_t)w * h, cudaMemcpyHostToDevice), "cudaMemcpy");
        uint32_t minw = 255;
        for (size_t i = 0; i < (size_t)w * h; ++i)
            if (weights[i] && weights[i] < minw) minw = weights[i];
        Pathfinding::set_board(d, w, h, Pathfinding::Position((uint16_t)tx, (uint16_t)ty), minw);
        auto r = a_star<Pathfinding::Position, 8, Pathfinding::neighbour_generator,
                        Pathfinding::admissible_heuristic>(Pathfinding::Position((uint16_t)sx, (uint16_t)sy),
                                                           Pathfinding::Position((uint16_t)tx, (uint16_t)ty), q);
        cudaFree(d);
        for (size_t i = 0; i < r.first.size(); ++i) out[i] = (uint32_t)r.first[i].y * w + r.first[i].x;
        return (int)r.first.size();
    } catch (...) {
        return -2;
    }
}

extern "C" int harness_line(uint32_t limit, uint32_t start, uint32_t target, uint32_t q, uint32_t* out) {
    try {
        gastar::plugin_host::check(cudaMemcpyToSymbol(line_limit, &limit, 4), "cudaMemcpyToSymbol");
        gastar::plugin_host::check(cudaMemcpyToSymbol(line_target, &target, 4), "cudaMemcpyToSymbol");
        auto r = a_star<Line, 3, line_gen, line_h>(Line{start}, Line{target}, q);
        for (size_t i = 0; i < r.first.size(); ++i) out[i] = r.first[i].v;
        return (int)r.first.size();
    } catch (...) {
        return -2;
    }
}

// SlidingPuzzle::solve / Pathfinding::solve on the reference's text input.
extern "C" int harness_solve_text(int grid, uint32_t n, const char* text, uint32_t q, char* out, size_t cap) {
    try {
        std::istringstream in(text);
        std::ostringstream o;
        if (grid) {
            auto r = Pathfinding::solve(in, q);
            for (auto& p : r.first) o << p << '\n';
        } else if (n == 3) {
            auto r = SlidingPuzzle::solve<3>(in, q);
            for (auto& p : r.first) o << p << '\n';
        } else if (n == 4) {
            auto r = SlidingPuzzle::solve<4>(in, q);
            for (auto& p : r.first) o << p << '\n';
        } else {
            auto r = SlidingPuzzle::solve<5>(in, q);
            for (auto& p : r.first) o << p << '\n';
        }
        const std::string s = o.str();
        if (s.size() + 1 > cap) return -3;
        std::memcpy(out, s.c_str(), s.size() + 1);
        return (int)s.size();
    } catch (...) {
        return -2;
    }
}
