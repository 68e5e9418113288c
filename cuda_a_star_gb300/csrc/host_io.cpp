// Host-side input/output of libgastar: the reference's text formats and the
// seeded synthetic instance generators.
//
// Text formats (reference michalborkowski96/cuda_a_star):
//   sliding : two whitespace-separated tokens, start then goal, each n*n
//             comma-separated integers with "_" or "0" for the blank
//             (Position(std::istream&), a_star_sliding_puzzle.h:21-48);
//             printed the same way with "_" for the blank (59-74).
//   grid    : "W,H" "sx,sy" "tx,ty" nObs ("x,y")*nObs nCost ("x,y,c")*nCost
//             (Pathfinding::solve and fill_generator_data,
//             a_star_pathfinding.h:223-231, 83-128); cells not listed cost 1;
//             a cell listed as an obstacle is impassable even if it also has
//             a cost; c is stored as an unsigned char like the reference
//             (value modulo 256).  Positions print as "x,y" (67-70).
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gastar.h"
#include "engine_internal.h"

namespace {

struct SplitMix64 {  // Steele, Lea, Flood 2014
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    uint32_t below(uint32_t n) { return (uint32_t)((next() >> 32) * (uint64_t)n >> 32); }
    double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// Whitespace-separated token reader over a C string.
struct Tokens {
    const char* p;
    bool next(std::string& out) {
        while (*p && std::isspace((unsigned char)*p)) ++p;
        if (!*p) return false;
        const char* b = p;
        while (*p && !std::isspace((unsigned char)*p)) ++p;
        out.assign(b, p);
        return true;
    }
};

bool parse_int(const std::string& s, long& v) {
    if (s.empty()) return false;
    char* end = nullptr;
    v = std::strtol(s.c_str(), &end, 10);
    return end && *end == '\0';
}

bool split_ints(const std::string& tok, std::vector<long>& out, size_t want, bool blank_ok) {
    out.clear();
    size_t b = 0;
    for (;;) {
        size_t e = tok.find(',', b);
        std::string f = tok.substr(b, e == std::string::npos ? std::string::npos : e - b);
        long v;
        if (blank_ok && f == "_") v = 0;
        else if (!parse_int(f, v)) return false;
        out.push_back(v);
        if (e == std::string::npos) break;
        b = e + 1;
    }
    return out.size() == want;
}

bool parse_board(const std::string& tok, uint32_t n, uint8_t* out) {
    std::vector<long> v;
    if (!split_ints(tok, v, (size_t)n * n, true)) return false;
    for (size_t i = 0; i < v.size(); ++i) {
        if (v[i] < 0 || v[i] >= (long)(n * n)) return false;
        out[i] = (uint8_t)v[i];
    }
    return gastar::valid_board(n, out);
}

}  // namespace

extern "C" {

int gastar_parse_sliding(const char* text, uint32_t n, uint8_t* start, uint8_t* goal) {
    if (!text || !start || !goal || n < 3 || n > 5) return GASTAR_BAD_INPUT;
    Tokens t{text};
    std::string a, b;
    if (!t.next(a) || !t.next(b)) {
        gastar::set_error("sliding: expected two boards");
        return GASTAR_BAD_INPUT;
    }
    if (!parse_board(a, n, start) || !parse_board(b, n, goal)) {
        gastar::set_error("sliding: a board is not a permutation of 0..n*n-1");
        return GASTAR_BAD_INPUT;
    }
    return GASTAR_OK;
}

int gastar_format_sliding(uint32_t n, const uint8_t* board, char* out, size_t cap) {
    if (!board || !out || n < 3 || n > 5) return GASTAR_BAD_INPUT;
    std::string s;
    for (uint32_t i = 0; i < n * n; ++i) {
        if (i) s += ',';
        s += board[i] ? std::to_string(board[i]) : std::string("_");
    }
    if (s.size() + 1 > cap) return GASTAR_PATH_CAP;
    std::memcpy(out, s.c_str(), s.size() + 1);
    return GASTAR_OK;
}

int gastar_parse_grid_dims(const char* text, uint32_t* w, uint32_t* h) {
    if (!text || !w || !h) return GASTAR_BAD_INPUT;
    Tokens t{text};
    std::string a;
    std::vector<long> v;
    if (!t.next(a) || !split_ints(a, v, 2, false) || v[0] <= 0 || v[1] <= 0 || v[0] > 65535 ||
        v[1] > 65535) {
        gastar::set_error("grid: expected board size W,H");
        return GASTAR_BAD_INPUT;
    }
    *w = (uint32_t)v[0];
    *h = (uint32_t)v[1];
    return GASTAR_OK;
}

int gastar_parse_grid(const char* text, uint32_t w, uint32_t h, uint8_t* weights, uint32_t* sx,
                      uint32_t* sy, uint32_t* tx, uint32_t* ty) {
    if (!text || !weights || !sx || !sy || !tx || !ty) return GASTAR_BAD_INPUT;
    Tokens t{text};
    std::string tok;
    std::vector<long> v;
    auto fail = [](const char* m) {
        gastar::set_error(std::string("grid: ") + m);
        return GASTAR_BAD_INPUT;
    };
    if (!t.next(tok) || !split_ints(tok, v, 2, false) || (uint32_t)v[0] != w || (uint32_t)v[1] != h)
        return fail("board size does not match");
    long pts[4];
    for (int k = 0; k < 2; ++k) {
        if (!t.next(tok) || !split_ints(tok, v, 2, false)) return fail("expected x,y");
        pts[2 * k] = v[0];
        pts[2 * k + 1] = v[1];
    }
    for (int k = 0; k < 2; ++k)
        if (pts[2 * k] < 0 || pts[2 * k] >= (long)w || pts[2 * k + 1] < 0 || pts[2 * k + 1] >= (long)h)
            return fail("start or target outside the board");
    *sx = (uint32_t)pts[0];
    *sy = (uint32_t)pts[1];
    *tx = (uint32_t)pts[2];
    *ty = (uint32_t)pts[3];
    const size_t cells = (size_t)w * h;
    std::memset(weights, 1, cells);
    std::vector<uint8_t> blocked(cells, 0);
    long cnt;
    if (!t.next(tok) || !parse_int(tok, cnt) || cnt < 0) return fail("expected obstacle count");
    for (long i = 0; i < cnt; ++i) {
        if (!t.next(tok) || !split_ints(tok, v, 2, false)) return fail("expected obstacle x,y");
        if (v[0] < 0 || v[0] >= (long)w || v[1] < 0 || v[1] >= (long)h) return fail("obstacle outside the board");
        blocked[(size_t)v[1] * w + (size_t)v[0]] = 1;
    }
    if (!t.next(tok) || !parse_int(tok, cnt) || cnt < 0) return fail("expected cost count");
    for (long i = 0; i < cnt; ++i) {
        if (!t.next(tok) || !split_ints(tok, v, 3, false)) return fail("expected cost x,y,c");
        if (v[0] < 0 || v[0] >= (long)w || v[1] < 0 || v[1] >= (long)h) return fail("cost cell outside the board");
        const uint8_t c = (uint8_t)((unsigned long)v[2] & 0xffu);
        if (c == 0) return fail("a cell cost of 0 (mod 256) is not supported");
        weights[(size_t)v[1] * w + (size_t)v[0]] = c;
    }
    for (size_t i = 0; i < cells; ++i)
        if (blocked[i]) weights[i] = 0;
    return GASTAR_OK;
}

// The reference's grid document for a dense weight array: obstacles are the
// cells of weight 0, costs the cells of weight other than 1 (the parser's
// default), each list in row-major order.
int gastar_format_grid(uint32_t w, uint32_t h, const uint8_t* weights, uint32_t sx, uint32_t sy, uint32_t tx,
                       uint32_t ty, char* out, size_t cap, size_t* written) {
    if (!weights || !written || w == 0 || h == 0 || sx >= w || tx >= w || sy >= h || ty >= h)
        return GASTAR_BAD_INPUT;
    const size_t cells = (size_t)w * h;
    size_t nobs = 0, ncost = 0;
    for (size_t i = 0; i < cells; ++i) {
        nobs += weights[i] == 0;
        ncost += weights[i] > 1;
    }
    std::string s;
    s.reserve(32 + nobs * 12 + ncost * 16);
    s += std::to_string(w) + ',' + std::to_string(h) + '\n';
    s += std::to_string(sx) + ',' + std::to_string(sy) + '\n';
    s += std::to_string(tx) + ',' + std::to_string(ty) + '\n';
    s += std::to_string(nobs) + '\n';
    for (size_t i = 0; i < cells; ++i)
        if (weights[i] == 0) s += std::to_string(i % w) + ',' + std::to_string(i / w) + '\n';
    s += std::to_string(ncost) + '\n';
    for (size_t i = 0; i < cells; ++i)
        if (weights[i] > 1)
            s += std::to_string(i % w) + ',' + std::to_string(i / w) + ',' + std::to_string(weights[i]) + '\n';
    *written = s.size() + 1;
    if (!out || s.size() + 1 > cap) return GASTAR_PATH_CAP;
    std::memcpy(out, s.c_str(), s.size() + 1);
    return GASTAR_OK;
}

namespace {
const uint8_t kGridMagic[8] = {'G', 'A', 'G', 'R', 'I', 'D', '1', 0};
void put_u32(uint8_t* p, uint32_t v) {
    for (int i = 0; i < 4; ++i) p[i] = (uint8_t)(v >> (8 * i));
}
uint32_t get_u32(const uint8_t* p) {
    return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24;
}
}  // namespace

int gastar_encode_grid_binary(uint32_t w, uint32_t h, const uint8_t* weights, uint32_t sx, uint32_t sy,
                              uint32_t tx, uint32_t ty, uint8_t* out, size_t cap, size_t* written) {
    if (!weights || !written || w == 0 || h == 0 || w > 65535 || h > 65535 || sx >= w || tx >= w || sy >= h ||
        ty >= h)
        return GASTAR_BAD_INPUT;
    const size_t cells = (size_t)w * h;
    *written = GASTAR_GRID_BINARY_HEADER + cells;
    if (!out || *written > cap) return GASTAR_PATH_CAP;
    std::memcpy(out, kGridMagic, 8);
    const uint32_t f[6] = {w, h, sx, sy, tx, ty};
    for (int i = 0; i < 6; ++i) put_u32(out + 8 + 4 * i, f[i]);
    std::memcpy(out + GASTAR_GRID_BINARY_HEADER, weights, cells);
    return GASTAR_OK;
}

int gastar_decode_grid_header(const uint8_t* buf, size_t len, uint32_t* w, uint32_t* h) {
    if (!buf || !w || !h || len < GASTAR_GRID_BINARY_HEADER || std::memcmp(buf, kGridMagic, 8) != 0) {
        gastar::set_error("binary grid: bad header");
        return GASTAR_BAD_INPUT;
    }
    *w = get_u32(buf + 8);
    *h = get_u32(buf + 12);
    if (*w == 0 || *h == 0 || *w > 65535 || *h > 65535) {
        gastar::set_error("binary grid: bad board size");
        return GASTAR_BAD_INPUT;
    }
    return GASTAR_OK;
}

int gastar_decode_grid_binary(const uint8_t* buf, size_t len, uint8_t* weights, size_t weights_cap, uint32_t* sx,
                              uint32_t* sy, uint32_t* tx, uint32_t* ty) {
    uint32_t w, h;
    const int rc = gastar_decode_grid_header(buf, len, &w, &h);
    if (rc != GASTAR_OK) return rc;
    if (!weights || !sx || !sy || !tx || !ty) return GASTAR_BAD_INPUT;
    const size_t cells = (size_t)w * h;
    if (len < GASTAR_GRID_BINARY_HEADER + cells) {
        gastar::set_error("binary grid: truncated");
        return GASTAR_BAD_INPUT;
    }
    if (weights_cap < cells) return GASTAR_PATH_CAP;
    *sx = get_u32(buf + 16);
    *sy = get_u32(buf + 20);
    *tx = get_u32(buf + 24);
    *ty = get_u32(buf + 28);
    if (*sx >= w || *tx >= w || *sy >= h || *ty >= h) {
        gastar::set_error("binary grid: start or target outside the board");
        return GASTAR_BAD_INPUT;
    }
    std::memcpy(weights, buf + GASTAR_GRID_BINARY_HEADER, cells);
    return GASTAR_OK;
}

// Seeded sliding-puzzle instance: goal = tiles 0..n*n-1 row-major (blank in
// cell 0); start = a random walk of L blank moves from the goal, L uniform in
// [walk_min, walk_max], never undoing the previous move.
int gastar_gen_sliding(uint32_t n, uint64_t seed, uint32_t walk_min, uint32_t walk_max, uint8_t* start,
                       uint8_t* goal) {
    if (n < 3 || n > 5 || !start || !goal || walk_min > walk_max) return GASTAR_BAD_INPUT;
    SplitMix64 r{seed};
    for (uint32_t i = 0; i < n * n; ++i) goal[i] = (uint8_t)i;
    std::memcpy(start, goal, n * n);
    const uint32_t len = walk_min + r.below(walk_max - walk_min + 1);
    int blank = 0, last = -1;
    static const int dr[4] = {1, -1, 0, 0}, dc[4] = {0, 0, 1, -1};
    for (uint32_t s = 0; s < len;) {
        const int m = (int)r.below(4);
        if (last >= 0 && m == (last ^ 1)) continue;  // no immediate reversal
        const int row = blank / (int)n + dr[m], col = blank % (int)n + dc[m];
        if (row < 0 || row >= (int)n || col < 0 || col >= (int)n) continue;
        const int q = row * (int)n + col;
        start[blank] = start[q];
        start[q] = 0;
        blank = q;
        last = m;
        ++s;
    }
    return GASTAR_OK;
}

// Seeded weighted grid: weights uniform in [wmin, wmax], each cell impassable
// (0) with probability `density`, then a random monotone corridor of
// right/down steps from (0,0) to (w-1,h-1) made passable so a path exists.
int gastar_gen_grid(uint32_t w, uint32_t h, uint64_t seed, double density, uint32_t wmin, uint32_t wmax,
                    uint8_t* weights) {
    if (!w || !h || !weights || wmin < 1 || wmax > 255 || wmin > wmax || density < 0 || density > 1)
        return GASTAR_BAD_INPUT;
    SplitMix64 r{seed};
    const uint32_t span = wmax - wmin + 1;
    const size_t cells = (size_t)w * h;
    for (size_t i = 0; i < cells; ++i) {
        const uint8_t wt = (uint8_t)(wmin + r.below(span));
        weights[i] = r.unit() < density ? 0 : wt;
    }
    uint32_t x = 0, y = 0;
    for (;;) {
        uint8_t& c = weights[(size_t)y * w + x];
        if (!c) c = (uint8_t)(wmin + r.below(span));
        if (x == w - 1 && y == h - 1) break;
        const bool right = (y == h - 1) || (x != w - 1 && (r.next() & 1));
        if (right) ++x;
        else ++y;
    }
    return GASTAR_OK;
}

}  // extern "C"
