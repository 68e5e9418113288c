// Golden-vector harness over the reference's own host-reachable functions.
//
// TEST INFRASTRUCTURE ONLY.  Built by `oracle/build.py --ref` from the reference
// headers where they lie (passed with -I); the binary goes to oracle/_ref/ and
// runs in the development container only.  It is how the oracle's
// restatement is pinned: tests/golden/make_golden.py runs it and stores its
// output as fixtures.
//
// The reference's successor and heuristic functions are `__device__` and read
// `__constant__` tables.  Compiled with `__device__` mapped to `__host__` and
// `__constant__` mapped to nothing, they become host functions over host
// globals, with their bodies unchanged.  a_star.h (kernels and the search
// loop) is kept out through its include guard and replaced by a declaration
// that is never called, so no kernel is instantiated.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <random>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#undef __device__
#define __device__ __host__
#undef __constant__
#define __constant__
#define A_STAR_H
#include "functional_types.h"
#include "helpers.h"
template <typename T, unsigned char max_neighbours, NeighbourGenerator<T> neighbour_generator,
          Heuristic<T> heuristic, uint16_t bucket_depth = 256>
std::pair<std::vector<T>, std::chrono::nanoseconds> a_star(const T&, const T&, const uint32_t) {
    std::fprintf(stderr, "a_star is not available in the host harness\n");
    std::abort();
}
#include "a_star_pathfinding.h"
#include "a_star_sliding_puzzle.h"

namespace {

template <unsigned char N>
std::string board_text(const std::vector<int>& cells) {
    std::string s;
    for (size_t i = 0; i < cells.size(); ++i) {
        if (i) s += ',';
        s += cells[i] ? std::to_string(cells[i]) : std::string("_");
    }
    return s;
}

template <unsigned char N>
void set_target(const SlidingPuzzle::Position<N>& target) {
    // Same table fill as set_manhattan_heuristic_target, written to the host
    // globals instead of through cudaMemcpyToSymbol.
    for (unsigned char i = 0; i < N; ++i)
        for (unsigned char j = 0; j < N; ++j) {
            SlidingPuzzle::manhattan_heuristic_data_x<N>[target.board[i][j]] = i;
            SlidingPuzzle::manhattan_heuristic_data_y<N>[target.board[i][j]] = j;
        }
}

template <unsigned char N>
std::string json_board(const SlidingPuzzle::Position<N>& p) {
    std::ostringstream o;
    o << '[';
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) o << (i || j ? "," : "") << int(p.board[i][j]);
    o << ']';
    return o.str();
}

// One JSON line per board: the reference's printer, heuristic and all four
// successor results.
template <unsigned char N>
void sliding_vectors(int count, uint64_t seed) {
    std::mt19937_64 rng(seed);
    std::vector<int> goal(N * N), cells(N * N);
    for (int i = 0; i < N * N; ++i) goal[i] = i;
    for (int c = 0; c < count; ++c) {
        if (c % 4 == 0) std::shuffle(goal.begin(), goal.end(), rng);
        for (int i = 0; i < N * N; ++i) cells[i] = i;
        std::shuffle(cells.begin(), cells.end(), rng);
        if (c < N * N) {  // every blank position at least once
            auto z = std::find(cells.begin(), cells.end(), 0) - cells.begin();
            std::swap(cells[z], cells[c]);
        }
        std::istringstream in(board_text<N>(cells) + " " + board_text<N>(goal));
        SlidingPuzzle::Position<N> s(in), t(in);
        set_target(t);
        std::ostringstream printed;
        printed << s;
        std::cout << "{\"kind\":\"sliding\",\"n\":" << int(N) << ",\"board\":" << json_board(s)
                  << ",\"goal\":" << json_board(t) << ",\"printed\":\"" << printed.str()
                  << "\",\"blank\":[" << int(s.pos_zero_x) << ',' << int(s.pos_zero_y)
                  << "],\"h_ref\":" << SlidingPuzzle::manhattan_heuristic<N>(s) << ",\"moves\":[";
        for (unsigned char m = 0; m < 4; ++m) {
            SlidingPuzzle::Position<N> d = s;
            bool ex = false;
            uint32_t cost = 0;
            SlidingPuzzle::neighbour_generator<N>(s, d, ex, cost, m);
            std::cout << (m ? "," : "") << "{\"exists\":" << (ex ? 1 : 0) << ",\"cost\":" << cost;
            if (ex) std::cout << ",\"next\":" << json_board(d);
            std::cout << '}';
        }
        std::cout << "]}\n";
    }
}

// Parses "start goal" pairs from stdin with the reference's Position parser
// and prints board, blank and printer output per board.
template <unsigned char N>
void sliding_parse() {
    std::string a, b;
    while (std::cin >> a >> b) {
        std::istringstream in(a + " " + b);
        SlidingPuzzle::Position<N> s(in), t(in);
        std::ostringstream ps, pt;
        ps << s;
        pt << t;
        std::cout << "{\"kind\":\"sliding_parse\",\"n\":" << int(N) << ",\"input\":[\"" << a
                  << "\",\"" << b << "\"],\"start\":" << json_board(s) << ",\"goal\":"
                  << json_board(t) << ",\"printed\":[\"" << ps.str() << "\",\"" << pt.str()
                  << "\"]}\n";
    }
}

std::vector<Pathfinding::Position> g_obstacles, g_cost_keys;
std::vector<unsigned char> g_cost_values;

// Random grids (sides <= 255, where the reference's 8-bit coordinates are
// exact): obstacle and cost lists sorted with the reference's own Position
// order, as fill_generator_data does, then every move from sampled cells.
void grid_vectors(int count, uint64_t seed) {
    std::mt19937_64 rng(seed);
    for (int c = 0; c < count; ++c) {
        uint16_t w = 1 + rng() % 40, h = 1 + rng() % 40;
        if (c == 0) w = h = 1;
        if (c == 1) { w = 255; h = 3; }
        if (c == 2) { w = 2; h = 255; }
        double dens = (rng() % 50) / 100.0, costd = (rng() % 100) / 100.0;
        g_obstacles.clear();
        g_cost_keys.clear();
        g_cost_values.clear();
        std::vector<std::tuple<uint16_t, uint16_t, uint16_t>> costs;
        std::vector<int> dense(size_t(w) * h, 1);
        for (uint16_t y = 0; y < h; ++y)
            for (uint16_t x = 0; x < w; ++x) {
                double u = (rng() >> 11) * (1.0 / 9007199254740992.0);
                if (u < dens) {
                    g_obstacles.emplace_back(x, y);
                    dense[size_t(y) * w + x] = 0;
                } else if ((rng() >> 11) * (1.0 / 9007199254740992.0) < costd) {
                    uint16_t cv = 1 + rng() % 9;
                    costs.emplace_back(x, y, cv);
                    dense[size_t(y) * w + x] = cv;
                }
            }
        std::sort(g_obstacles.begin(), g_obstacles.end());
        std::sort(costs.begin(), costs.end(), [](const auto& a, const auto& b) {
            return Pathfinding::Position(std::get<0>(a), std::get<1>(a)) <
                   Pathfinding::Position(std::get<0>(b), std::get<1>(b));
        });
        for (auto& t : costs) {
            g_cost_keys.emplace_back(std::get<0>(t), std::get<1>(t));
            g_cost_values.push_back(std::get<2>(t));
        }
        Pathfinding::neighbour_generator_board_size = Pathfinding::Position(w, h);
        Pathfinding::neighbour_generator_obstacles = g_obstacles.data();
        Pathfinding::neighbour_generator_obstacles_size = g_obstacles.size();
        Pathfinding::neighbour_generator_costs_keys = g_cost_keys.data();
        Pathfinding::neighbour_generator_costs_values = g_cost_values.data();
        Pathfinding::neighbour_generator_costs_size = g_cost_keys.size();
        Pathfinding::Position target(rng() % w, rng() % h);
        Pathfinding::manhattan_heuristic_data = target;
        std::cout << "{\"kind\":\"grid\",\"w\":" << w << ",\"h\":" << h << ",\"weights\":[";
        for (size_t i = 0; i < dense.size(); ++i) std::cout << (i ? "," : "") << dense[i];
        std::cout << "],\"target\":[" << target.x << ',' << target.y << "],\"cells\":[";
        int samples = std::min<int>(24, w * h);
        for (int s = 0; s < samples; ++s) {
            Pathfinding::Position src(rng() % w, rng() % h);
            if (s == 0) src = Pathfinding::Position(0, 0);
            if (s == 1) src = Pathfinding::Position(w - 1, h - 1);
            std::cout << (s ? "," : "") << "{\"x\":" << src.x << ",\"y\":" << src.y
                      << ",\"h_ref\":" << Pathfinding::manhattan_heuristic(src) << ",\"moves\":[";
            for (unsigned char m = 0; m < 8; ++m) {
                Pathfinding::Position d(0, 0);
                bool ex = false;
                uint32_t cost = 0;
                Pathfinding::neighbour_generator(src, d, ex, cost, m);
                std::cout << (m ? "," : "") << "{\"exists\":" << (ex ? 1 : 0);
                if (ex) std::cout << ",\"x\":" << d.x << ",\"y\":" << d.y << ",\"cost\":" << cost;
                std::cout << '}';
            }
            std::cout << "]}";
        }
        std::cout << "]}\n";
    }
}

// Parses one grid-format document from stdin with the reference's token
// readers (a_star_pathfinding.h:38-65, 83-128) and prints what it read.
void grid_parse() {
    Pathfinding::Position board(std::cin), start(std::cin), target(std::cin);
    int32_t obstacle_count;
    std::cin >> obstacle_count;
    std::vector<Pathfinding::Position> obstacles;
    for (int32_t i = 0; i < obstacle_count; ++i) obstacles.emplace_back(std::cin);
    std::sort(obstacles.begin(), obstacles.end());
    int32_t cost_count;
    std::cin >> cost_count;
    std::vector<std::tuple<uint16_t, uint16_t, uint16_t>> costs;
    for (int32_t i = 0; i < cost_count; ++i) costs.push_back(Pathfinding::scan_triple_int(std::cin));
    std::ostringstream pb, ps, pt;
    pb << board;
    ps << start;
    pt << target;
    std::cout << "{\"kind\":\"grid_parse\",\"board\":\"" << pb.str() << "\",\"start\":\"" << ps.str()
              << "\",\"target\":\"" << pt.str() << "\",\"obstacles\":[";
    for (size_t i = 0; i < obstacles.size(); ++i)
        std::cout << (i ? "," : "") << '[' << obstacles[i].x << ',' << obstacles[i].y << ']';
    std::cout << "],\"costs\":[";
    for (size_t i = 0; i < costs.size(); ++i)
        std::cout << (i ? "," : "") << '[' << std::get<0>(costs[i]) << ',' << std::get<1>(costs[i])
                  << ',' << int((unsigned char)std::get<2>(costs[i])) << ']';
    std::cout << "]}\n";
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr,
                     "usage: ref_harness sliding N COUNT SEED | grid COUNT SEED | "
                     "parse_sliding N | parse_grid\n");
        return 2;
    }
    std::string mode = argv[1];
    if (mode == "sliding" && argc == 5) {
        int n = std::atoi(argv[2]), count = std::atoi(argv[3]);
        uint64_t seed = std::strtoull(argv[4], nullptr, 10);
        if (n == 3) sliding_vectors<3>(count, seed);
        else if (n == 4) sliding_vectors<4>(count, seed);
        else if (n == 5) sliding_vectors<5>(count, seed);
        else return 2;
    } else if (mode == "parse_sliding" && argc == 3) {
        int n = std::atoi(argv[2]);
        if (n == 3) sliding_parse<3>();
        else if (n == 4) sliding_parse<4>();
        else if (n == 5) sliding_parse<5>();
        else return 2;
    } else if (mode == "grid" && argc == 4) {
        grid_vectors(std::atoi(argv[2]), std::strtoull(argv[3], nullptr, 10));
    } else if (mode == "parse_grid") {
        grid_parse();
    } else {
        return 2;
    }
    return 0;
}
