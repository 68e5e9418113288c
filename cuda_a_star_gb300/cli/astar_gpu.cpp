// astar_gpu: command-line front end with the reference's interface
// (main.cu:31-77): --version sliding|pathfinding, --input-data FILE,
// --output-data FILE (stdin/stdout when omitted); prints the search time in
// whole milliseconds, then the path one state per line (empty when there is
// none).  Bad flags print a message and exit with -1 like main.cu:20-24.
//
// Additions: --size 3|4|5 (sliding; default: from the input, where the
// reference always used 5, main.cu:72), --queues Q (default 4096 like
// NUM_QUEUES, main.cu:18), --device D (main.cu:17 fixed device 1),
// --heuristic admissible|reference|zero, --moves standard|reference,
// --delta D (pop window); pathfinding only: --input-format text|binary (the
// binary dense grid of gastar_encode_grid_binary) and --convert text|binary
// (write the input grid in that format to the output and exit, no GPU).
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "gastar.h"

namespace {

[[noreturn]] void error(const std::string& msg) {
    std::cout << msg << std::endl;
    std::exit(-1);
}

uint32_t parse_u32(const std::string& flag, const std::string& v) {
    char* end = nullptr;
    const unsigned long x = std::strtoul(v.c_str(), &end, 10);
    if (!end || *end) error("Bad value for " + flag + ": " + v);
    return (uint32_t)x;
}

}  // namespace

int main(int argc, char** argv) {
    std::string input, output, version, in_format = "text", convert;
    uint32_t size = 0, queues = 4096, delta = 0;
    int device = 0;
    gastar_config cfg;
    gastar_config_default(&cfg);
    for (int i = 1; i < argc; i += 2) {
        if (i == argc - 1) error("Parameter without argument.");
        const std::string f = argv[i], v = argv[i + 1];
        if (f == "--version") version = v;
        else if (f == "--input-data") input = v;
        else if (f == "--output-data") output = v;
        else if (f == "--size") size = parse_u32(f, v);
        else if (f == "--queues") queues = parse_u32(f, v);
        else if (f == "--device") device = (int)parse_u32(f, v);
        else if (f == "--delta") delta = parse_u32(f, v);
        else if (f == "--input-format") {
            if (v != "text" && v != "binary") error("Unknown input format " + v);
            in_format = v;
        } else if (f == "--convert") {
            if (v != "text" && v != "binary") error("Unknown output format " + v);
            convert = v;
        }
        else if (f == "--heuristic") {
            if (v == "admissible") cfg.heuristic = GASTAR_H_ADMISSIBLE;
            else if (v == "reference") cfg.heuristic = GASTAR_H_REFERENCE;
            else if (v == "zero") cfg.heuristic = GASTAR_H_ZERO;
            else error("Unknown heuristic " + v);
        } else if (f == "--moves") {
            if (v == "standard") cfg.moves = GASTAR_MOVES_STANDARD;
            else if (v == "reference") cfg.moves = GASTAR_MOVES_REFERENCE;
            else error("Unknown moves " + v);
        } else error("Unknown option " + f);
    }
    if (version != "sliding" && version != "pathfinding") error("Unknown version " + version);
    std::string text;
    {
        std::stringstream ss;
        if (input.empty()) ss << std::cin.rdbuf();
        else {
            std::ifstream in(input, std::ios::binary);
            if (!in) error("Cannot open " + input);
            ss << in.rdbuf();
        }
        text = ss.str();
    }
    if ((in_format == "binary" || !convert.empty()) && version != "pathfinding")
        error("--input-format binary and --convert apply to pathfinding only.");
    // The grid, from either format.
    uint32_t w = 0, h = 0, sx = 0, sy = 0, tx = 0, ty = 0;
    std::vector<uint8_t> wts;
    if (version == "pathfinding") {
        if (in_format == "binary") {
            const uint8_t* b = reinterpret_cast<const uint8_t*>(text.data());
            if (gastar_decode_grid_header(b, text.size(), &w, &h) != GASTAR_OK) error(gastar_last_error());
            wts.resize((size_t)w * h);
            if (gastar_decode_grid_binary(b, text.size(), wts.data(), wts.size(), &sx, &sy, &tx, &ty) != GASTAR_OK)
                error(gastar_last_error());
        } else {
            if (gastar_parse_grid_dims(text.c_str(), &w, &h) != GASTAR_OK) error(gastar_last_error());
            wts.resize((size_t)w * h);
            if (gastar_parse_grid(text.c_str(), w, h, wts.data(), &sx, &sy, &tx, &ty) != GASTAR_OK)
                error(gastar_last_error());
        }
    }
    if (!convert.empty()) {
        size_t n = 0;
        std::string bytes;
        if (convert == "binary") {
            bytes.resize(GASTAR_GRID_BINARY_HEADER + wts.size());
            if (gastar_encode_grid_binary(w, h, wts.data(), sx, sy, tx, ty, reinterpret_cast<uint8_t*>(&bytes[0]),
                                          bytes.size(), &n) != GASTAR_OK)
                error("Cannot encode the grid.");
        } else {
            gastar_format_grid(w, h, wts.data(), sx, sy, tx, ty, nullptr, 0, &n);
            bytes.resize(n);
            if (gastar_format_grid(w, h, wts.data(), sx, sy, tx, ty, &bytes[0], bytes.size(), &n) != GASTAR_OK)
                error("Cannot format the grid.");
            bytes.resize(n - 1);  // without the NUL
        }
        if (output.empty()) std::cout.write(bytes.data(), (std::streamsize)bytes.size());
        else {
            std::ofstream o(output, std::ios::binary);
            if (!o) error("Cannot open " + output);
            o.write(bytes.data(), (std::streamsize)bytes.size());
        }
        return 0;
    }
    cfg.num_queues = queues;
    cfg.delta = delta;
    gastar_ctx* ctx = gastar_create(device);
    if (!ctx) error(std::string("CUDA: ") + gastar_last_error());
    std::ostringstream out;
    gastar_result r;
    if (version == "sliding") {
        if (!size) {  // tiles in the first token
            std::istringstream t(text);
            std::string tok;
            t >> tok;
            const size_t cells = (size_t)std::count(tok.begin(), tok.end(), ',') + 1;
            size = cells == 9 ? 3 : cells == 16 ? 4 : cells == 25 ? 5 : 0;
            if (!size) error("Sliding puzzle incorrect input.");
        }
        std::vector<uint8_t> s(size * size), g(size * size), path((size_t)4096 * size * size);
        if (gastar_parse_sliding(text.c_str(), size, s.data(), g.data()) != GASTAR_OK)
            error(gastar_last_error());
        if (gastar_solve_sliding(ctx, size, s.data(), g.data(), &cfg, path.data(), 4096, &r) != GASTAR_OK)
            error(gastar_last_error());
        out << (long long)r.kernel_ms << '\n';
        char line[256];
        for (uint32_t i = 0; r.status == GASTAR_OK && i < r.path_len; ++i) {
            gastar_format_sliding(size, path.data() + (size_t)i * size * size, line, sizeof(line));
            out << line << '\n';
        }
    } else {
        std::vector<uint32_t> path((size_t)w * h);
        if (gastar_solve_grid(ctx, w, h, wts.data(), sx, sy, tx, ty, &cfg, path.data(), (uint32_t)path.size(),
                              &r) != GASTAR_OK)
            error(gastar_last_error());
        out << (long long)r.kernel_ms << '\n';
        for (uint32_t i = 0; r.status == GASTAR_OK && i < r.path_len; ++i)
            out << path[i] % w << ',' << path[i] / w << '\n';
    }
    gastar_destroy(ctx);
    if (output.empty()) std::cout << out.str();
    else {
        std::ofstream o(output);
        if (!o) error("Cannot open " + output);
        o << out.str();
    }
    return 0;
}
