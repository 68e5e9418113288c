// The reference's front ends on this engine: SlidingPuzzle:: and
// Pathfinding:: with the same state layouts, plugin functions, input parsing,
// printing and solve() signatures as a_star_sliding_puzzle.h and
// a_star_pathfinding.h of michalborkowski96/cuda_a_star.
//
//  * Position types keep the reference's byte layout (a_star_sliding_puzzle.h:13-19,
//    a_star_pathfinding.h:17-36), so they also work as plugin states of the
//    generic ::a_star template (include/gastar/a_star.cuh).
//  * neighbour_generator: the four blank moves (row+1, row-1, col+1, col-1) with
//    cost 1; defining GASTAR_REFERENCE_MOVES before including this header keeps
//    the reference's arithmetic, under which only moves 0 and 2 exist
//    (a_star_sliding_puzzle.h:106-111).  The grid generator reads a dense
//    weight grid (0 = impassable) from device memory set by set_board().
//  * manhattan_heuristic: the reference's formulas (blank included; Manhattan
//    on 8-connected grids -- not admissible); admissible_* variants give
//    optimal paths.
//  * solve(): parses the reference's text input and runs the engine's
//    specialised kernels through the C ABI (libgastar.so) with the admissible
//    heuristics; returns the path and the search time like the reference.
#pragma once

#include <cstdint>
#include <istream>
#include <ostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../gastar.h"
#include "a_star.cuh"

namespace gastar_ref_detail {
inline gastar_ctx* context() {
    static gastar_ctx* c = gastar_create(-1);
    if (!c) throw std::runtime_error(gastar_last_error());
    return c;
}
inline std::string read_all(std::istream& in) {
    std::stringstream ss;
    ss << in.rdbuf();
    return ss.str();
}
}  // namespace gastar_ref_detail

namespace SlidingPuzzle {

template <unsigned char size> struct Position {
    unsigned char pos_zero_x;
    unsigned char pos_zero_y;
    unsigned char board[size][size];
    unsigned char padding[(4 - ((size * size + 2) % 4)) % 4];

    __host__ __device__ Position() = delete;
    // Reads one token of size*size comma-separated tiles, "_" or "0" = blank.
    __host__ explicit Position(std::istream& in) {
        std::string tok;
        in >> tok;
        std::vector<int> v;
        size_t b = 0;
        for (;;) {
            const size_t e = tok.find(',', b);
            const std::string f = tok.substr(b, e == std::string::npos ? std::string::npos : e - b);
            v.push_back(f == "_" ? 0 : std::stoi(f));
            if (e == std::string::npos) break;
            b = e + 1;
        }
        if (v.size() != (size_t)size * size) throw std::runtime_error("Sliding puzzle incorrect input.");
        for (int i = 0; i < size; ++i)
            for (int j = 0; j < size; ++j) {
                board[i][j] = (unsigned char)v[i * size + j];
                if (!board[i][j]) {
                    pos_zero_x = (unsigned char)i;
                    pos_zero_y = (unsigned char)j;
                }
            }
        for (unsigned i = 0; i < sizeof(padding); ++i) padding[i] = 69;
    }
    __host__ explicit Position(const uint8_t* cells) {
        for (int i = 0; i < size; ++i)
            for (int j = 0; j < size; ++j) {
                board[i][j] = cells[i * size + j];
                if (!board[i][j]) {
                    pos_zero_x = (unsigned char)i;
                    pos_zero_y = (unsigned char)j;
                }
            }
        for (unsigned i = 0; i < sizeof(padding); ++i) padding[i] = 69;
    }
    __host__ __device__ bool operator==(const Position& o) const {
        const unsigned char* a = reinterpret_cast<const unsigned char*>(this);
        const unsigned char* b = reinterpret_cast<const unsigned char*>(&o);
        for (unsigned i = 0; i < sizeof(Position); ++i)
            if (a[i] != b[i]) return false;
        return true;
    }
    __host__ __device__ bool operator<(const Position& o) const {
        const unsigned char* a = reinterpret_cast<const unsigned char*>(this);
        const unsigned char* b = reinterpret_cast<const unsigned char*>(&o);
        for (unsigned i = 0; i < sizeof(Position); ++i)
            if (a[i] != b[i]) return a[i] < b[i];
        return false;
    }
};

template <unsigned char size> std::ostream& operator<<(std::ostream& o, const Position<size>& p) {
    for (int i = 0; i < size; ++i)
        for (int j = 0; j < size; ++j) {
            if (p.board[i][j]) o << (int)p.board[i][j];
            else o << '_';
            if (i != size - 1 || j != size - 1) o << ',';
        }
    return o;
}

template <unsigned char size>
__device__ void neighbour_generator(const Position<size>& source, Position<size>& target,
                                    bool& target_exists, uint32_t& cost, unsigned char i) {
    cost = 1;
    int r = source.pos_zero_x, c = source.pos_zero_y;
#ifdef GASTAR_REFERENCE_MOVES
    if (i == 1 || i == 3) {  // the reference's uint16 sum never wraps below size
        target_exists = false;
        return;
    }
#endif
    const int nr = r + (i == 0 ? 1 : i == 1 ? -1 : 0), nc = c + (i == 2 ? 1 : i == 3 ? -1 : 0);
    if (nr < 0 || nc < 0 || nr >= size || nc >= size) {
        target_exists = false;
        return;
    }
    target_exists = true;
    target = source;
    target.board[r][c] = source.board[nr][nc];
    target.board[nr][nc] = 0;
    target.pos_zero_x = (unsigned char)nr;
    target.pos_zero_y = (unsigned char)nc;
}

// Goal row/column of every tile value, set by set_manhattan_heuristic_target.
template <unsigned char size> __constant__ signed char manhattan_target_row[size * size];
template <unsigned char size> __constant__ signed char manhattan_target_col[size * size];

template <unsigned char size> __host__ void set_manhattan_heuristic_target(const Position<size>& target) {
    signed char r[size * size], c[size * size];
    for (int i = 0; i < size; ++i)
        for (int j = 0; j < size; ++j) {
            r[target.board[i][j]] = (signed char)i;
            c[target.board[i][j]] = (signed char)j;
        }
    gastar::plugin_host::check(cudaMemcpyToSymbol(manhattan_target_row<size>, r, sizeof(r)), "cudaMemcpyToSymbol");
    gastar::plugin_host::check(cudaMemcpyToSymbol(manhattan_target_col<size>, c, sizeof(c)), "cudaMemcpyToSymbol");
}

template <unsigned char size, bool with_blank> __device__ uint32_t manhattan_sum(const Position<size>& p) {
    uint32_t s = 0;
    for (int i = 0; i < size; ++i)
        for (int j = 0; j < size; ++j) {
            const unsigned char t = p.board[i][j];
            if (!with_blank && t == 0) continue;
            const int dr = manhattan_target_row<size>[t] - i, dc = manhattan_target_col<size>[t] - j;
            s += (uint32_t)((dr < 0 ? -dr : dr) + (dc < 0 ? -dc : dc));
        }
    return s;
}
// The reference's formula: every cell, the blank included (not admissible).
template <unsigned char size> __device__ uint32_t manhattan_heuristic(const Position<size>& p) {
    return manhattan_sum<size, true>(p);
}
template <unsigned char size> __device__ uint32_t admissible_manhattan_heuristic(const Position<size>& p) {
    return manhattan_sum<size, false>(p);
}

// solve<size>(in, num_queues): start and goal boards from `in`; the engine's
// specialised kernel, admissible heuristic, four moves.
template <unsigned char size>
std::pair<std::vector<Position<size>>, std::chrono::nanoseconds> solve(std::istream& in, uint32_t num_queues) {
    const std::string text = gastar_ref_detail::read_all(in);
    uint8_t s[size * size], g[size * size];
    if (gastar_parse_sliding(text.c_str(), size, s, g) != GASTAR_OK) throw std::runtime_error(gastar_last_error());
    gastar_config cfg;
    gastar_config_default(&cfg);
    cfg.num_queues = num_queues;
    std::vector<uint8_t> path((size_t)4096 * size * size);
    gastar_result r;
    if (gastar_solve_sliding(gastar_ref_detail::context(), size, s, g, &cfg, path.data(), 4096, &r) != GASTAR_OK)
        throw std::runtime_error(gastar_last_error());
    std::vector<Position<size>> out;
    if (r.status == GASTAR_OK)
        for (uint32_t i = 0; i < r.path_len; ++i) out.emplace_back(path.data() + (size_t)i * size * size);
    return {out, std::chrono::nanoseconds((long long)((double)r.kernel_ms * 1e6))};
}

}  // namespace SlidingPuzzle

namespace Pathfinding {

struct Position {
    uint16_t x;
    uint16_t y;
    Position() = default;
    __host__ __device__ Position(uint16_t x, uint16_t y) : x(x), y(y) {}
    // Reads one "x,y" token.
    __host__ explicit Position(std::istream& in) {
        std::string tok;
        in >> tok;
        const size_t d = tok.find(',');
        if (d == std::string::npos) throw std::runtime_error("Pathfinding incorrect input.");
        x = (uint16_t)std::stoi(tok.substr(0, d));
        y = (uint16_t)std::stoi(tok.substr(d + 1));
    }
    __host__ __device__ bool operator==(const Position& o) const { return x == o.x && y == o.y; }
    __host__ __device__ bool operator<(const Position& o) const { return y != o.y ? y < o.y : x < o.x; }
};

inline std::ostream& operator<<(std::ostream& o, const Position& p) {
    o << p.x << ',' << p.y;
    return o;
}

// Board data read by the plugin functions (device memory, set by set_board).
__constant__ const uint8_t* board_weights;
__constant__ uint32_t board_w, board_h;
__constant__ uint16_t target_x, target_y;
__constant__ uint32_t board_min_weight;

// Dense weights (w*h bytes on the device, index y*w + x, 0 = impassable).
__host__ inline void set_board(const uint8_t* d_weights, uint32_t w, uint32_t h, Position target,
                               uint32_t min_weight) {
    using gastar::plugin_host::check;
    check(cudaMemcpyToSymbol(board_weights, &d_weights, sizeof(d_weights)), "cudaMemcpyToSymbol");
    check(cudaMemcpyToSymbol(board_w, &w, sizeof(w)), "cudaMemcpyToSymbol");
    check(cudaMemcpyToSymbol(board_h, &h, sizeof(h)), "cudaMemcpyToSymbol");
    check(cudaMemcpyToSymbol(target_x, &target.x, sizeof(target.x)), "cudaMemcpyToSymbol");
    check(cudaMemcpyToSymbol(target_y, &target.y, sizeof(target.y)), "cudaMemcpyToSymbol");
    check(cudaMemcpyToSymbol(board_min_weight, &min_weight, sizeof(min_weight)), "cudaMemcpyToSymbol");
}

// 8 moves in the reference's order (a_star_pathfinding.h:150-183); the cost
// is the entered cell's weight.
__device__ inline void neighbour_generator(const Position& source, Position& target, bool& target_exists,
                                           uint32_t& cost, unsigned char i) {
    const int dx = (i == 0 || i == 4 || i == 5) ? 1 : (i == 1 || i == 6 || i == 7) ? -1 : 0;
    const int dy = (i == 2 || i == 4 || i == 6) ? 1 : (i == 3 || i == 5 || i == 7) ? -1 : 0;
    const int nx = source.x + dx, ny = source.y + dy;
    if (nx < 0 || ny < 0 || nx >= (int)board_w || ny >= (int)board_h) {
        target_exists = false;
        return;
    }
    const uint8_t wt = board_weights[(size_t)ny * board_w + nx];
    if (!wt) {
        target_exists = false;
        return;
    }
    target_exists = true;
    target.x = (uint16_t)nx;
    target.y = (uint16_t)ny;
    cost = wt;
}

// The reference's heuristic (a_star_pathfinding.h:219-221, not admissible).
__device__ inline uint32_t manhattan_heuristic(const Position& p) {
    const int dx = (int)target_x - p.x, dy = (int)target_y - p.y;
    return (uint32_t)((dx < 0 ? -dx : dx) + (dy < 0 ? -dy : dy));
}
// Chebyshev distance x minimum weight: admissible for 8-connected moves.
__device__ inline uint32_t admissible_heuristic(const Position& p) {
    const int dx = (int)target_x - p.x, dy = (int)target_y - p.y;
    const uint32_t ax = (uint32_t)(dx < 0 ? -dx : dx), ay = (uint32_t)(dy < 0 ? -dy : dy);
    return (ax > ay ? ax : ay) * board_min_weight;
}

// solve(in, num_queues): the reference's grid document; the engine's dense
// grid kernel with the admissible heuristic.
inline std::pair<std::vector<Position>, std::chrono::nanoseconds> solve(std::istream& in, uint32_t num_queues) {
    const std::string text = gastar_ref_detail::read_all(in);
    uint32_t w, h, sx, sy, tx, ty;
    if (gastar_parse_grid_dims(text.c_str(), &w, &h) != GASTAR_OK) throw std::runtime_error(gastar_last_error());
    std::vector<uint8_t> wts((size_t)w * h);
    if (gastar_parse_grid(text.c_str(), w, h, wts.data(), &sx, &sy, &tx, &ty) != GASTAR_OK)
        throw std::runtime_error(gastar_last_error());
    gastar_config cfg;
    gastar_config_default(&cfg);
    cfg.num_queues = num_queues;
    cfg.delta = 36;
    std::vector<uint32_t> path((size_t)w * h);
    gastar_result r;
    if (gastar_solve_grid(gastar_ref_detail::context(), w, h, wts.data(), sx, sy, tx, ty, &cfg, path.data(),
                          (uint32_t)path.size(), &r) != GASTAR_OK)
        throw std::runtime_error(gastar_last_error());
    std::vector<Position> out;
    if (r.status == GASTAR_OK)
        for (uint32_t i = 0; i < r.path_len; ++i) out.emplace_back((uint16_t)(path[i] % w), (uint16_t)(path[i] / w));
    return {out, std::chrono::nanoseconds((long long)((double)r.kernel_ms * 1e6))};
}

}  // namespace Pathfinding
