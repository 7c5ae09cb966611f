// Edge-list reader for the reference's input format (src/input/GraphInputIterator.cpp:3-36):
// the first line is skipped unconditionally, then `n m` (unsigned), then m triples `u v w`
// read as unsigned, separated by any whitespace. The reference throws through ifstream
// failbits on malformed input (GraphInputIterator.hpp:19); here the reader returns
// CAC_ERR_IO / CAC_ERR_PARSE with a message instead.
//
// The triples are parsed by all host threads at once: the body is split into chunks at
// whitespace, a first pass counts the tokens of every chunk, and the second pass converts
// each chunk straight into the caller's arrays at its token offset.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "cac_internal.h"

namespace cac {
namespace {

inline bool is_space(char c) { return c == ' ' || c == '\n' || c == '\t' || c == '\r' || c == '\f' || c == '\v'; }

struct FileBuf {
    std::vector<char> data;
};

int read_all(const char *path, FileBuf &fb) {
    FILE *f = std::fopen(path, "rb");
    if (!f) {
        set_error(std::string("cannot open ") + path);
        return CAC_ERR_IO;
    }
    std::fseek(f, 0, SEEK_END);
    long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (size < 0) {
        std::fclose(f);
        set_error(std::string("cannot size ") + path);
        return CAC_ERR_IO;
    }
    fb.data.resize((size_t)size + 1);
    size_t got = size ? std::fread(fb.data.data(), 1, (size_t)size, f) : 0;
    std::fclose(f);
    if (got != (size_t)size) {
        set_error(std::string("short read of ") + path);
        return CAC_ERR_IO;
    }
    fb.data[(size_t)size] = '\0';
    fb.data.resize((size_t)size);
    return CAC_OK;
}

// Parses one unsigned token at p (p < end, not whitespace); returns false on junk/overflow.
inline bool parse_u32(const char *&p, const char *end, uint32_t &out) {
    uint64_t x = 0;
    const char *s = p;
    if (p < end && *p == '+') p++;
    const char *digits = p;
    while (p < end && *p >= '0' && *p <= '9') {
        x = x * 10 + (uint64_t)(*p - '0');
        if (x > 0xFFFFFFFFull) return false;
        p++;
    }
    if (p == digits || (p < end && !is_space(*p))) {
        p = s;
        return false;
    }
    out = (uint32_t)x;
    return true;
}

// Positions just past the header: skip line 1, then read n and m.
int parse_header_buf(const char *b, const char *end, uint32_t *n, uint64_t *m, const char **body) {
    const char *p = (const char *)std::memchr(b, '\n', (size_t)(end - b));
    if (!p) {
        set_error("input has no header line");
        return CAC_ERR_PARSE;
    }
    p++;
    uint32_t vals[2];
    for (int k = 0; k < 2; k++) {
        while (p < end && is_space(*p)) p++;
        if (p >= end || !parse_u32(p, end, vals[k])) {
            set_error("cannot read the vertex / edge counts");
            return CAC_ERR_PARSE;
        }
    }
    *n = vals[0];
    *m = vals[1];
    *body = p;
    return CAC_OK;
}

}  // namespace
}  // namespace cac

using namespace cac;

extern "C" {

int cac_parse_header(const char *path, uint32_t *n, uint64_t *m) {
    if (!path || !n || !m) { set_error("cac_parse_header: invalid argument"); return CAC_ERR_INVALID; }
    FILE *f = std::fopen(path, "rb");
    if (!f) { set_error(std::string("cannot open ") + path); return CAC_ERR_IO; }
    std::vector<char> head(1 << 16);
    size_t got = std::fread(head.data(), 1, head.size(), f);
    // the first line may be long: keep reading until the counts are in the buffer
    while (got == head.size()) {
        const char *nl = (const char *)std::memchr(head.data(), '\n', got);
        if (nl && (size_t)(nl - head.data()) + 64 < got) break;
        head.resize(head.size() * 2);
        got += std::fread(head.data() + got, 1, head.size() - got, f);
    }
    std::fclose(f);
    const char *body;
    return parse_header_buf(head.data(), head.data() + got, n, m, &body);
}

int cac_parse_file(const char *path, uint32_t *n, uint64_t *m, uint32_t *u, uint32_t *v, uint32_t *w,
                   uint64_t capacity) {
    if (!path || !n || !m) { set_error("cac_parse_file: invalid argument"); return CAC_ERR_INVALID; }
    FileBuf fb;
    CAC_TRY(read_all(path, fb));
    const char *b = fb.data.data(), *end = b + fb.data.size();
    const char *body;
    CAC_TRY(parse_header_buf(b, end, n, m, &body));
    const uint64_t edges = *m;
    if (edges > capacity || (edges && (!u || !v))) {
        set_error("cac_parse_file: output capacity " + std::to_string(capacity) + " < edge count " +
                  std::to_string(edges));
        return CAC_ERR_INVALID;
    }
    const uint64_t need = 3 * edges;
    // chunk boundaries at whitespace
    unsigned T = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const size_t len = (size_t)(end - body);
    if (len < (1u << 20)) T = 1;
    std::vector<const char *> cut(T + 1);
    cut[0] = body;
    cut[T] = end;
    for (unsigned t = 1; t < T; t++) {
        const char *q = body + len * t / T;
        while (q < end && !is_space(*q)) q++;
        cut[t] = std::max(q, cut[t - 1]);
    }
    std::vector<uint64_t> tokens(T + 1, 0);
    auto count = [&](unsigned t) {
        uint64_t c = 0;
        const char *p = cut[t], *e = cut[t + 1];
        while (p < e) {
            while (p < e && is_space(*p)) p++;
            if (p >= e) break;
            c++;
            while (p < e && !is_space(*p)) p++;
        }
        tokens[t + 1] = c;
    };
    std::vector<std::thread> th;
    for (unsigned t = 1; t < T; t++) th.emplace_back(count, t);
    count(0);
    for (auto &x : th) x.join();
    th.clear();
    for (unsigned t = 0; t < T; t++) tokens[t + 1] += tokens[t];
    if (tokens[T] < need) {
        set_error("input declares " + std::to_string(edges) + " edges but holds only " +
                  std::to_string(tokens[T] / 3) + " complete lines");
        return CAC_ERR_PARSE;
    }
    std::vector<int> bad(T, 0);
    auto conv = [&](unsigned t) {
        uint64_t k = tokens[t];
        const char *p = cut[t], *e = cut[t + 1];
        while (p < e && k < need) {
            while (p < e && is_space(*p)) p++;
            if (p >= e) break;
            uint32_t x;
            if (!parse_u32(p, e, x)) { bad[t] = 1; return; }
            const uint64_t edge = k / 3;
            switch (k % 3) {
                case 0: u[edge] = x; break;
                case 1: v[edge] = x; break;
                default: if (w) w[edge] = x; break;
            }
            k++;
        }
    };
    for (unsigned t = 1; t < T; t++) th.emplace_back(conv, t);
    conv(0);
    for (auto &x : th) x.join();
    for (unsigned t = 0; t < T; t++)
        if (bad[t]) { set_error("non-numeric or out-of-range token in the edge list"); return CAC_ERR_PARSE; }
    for (uint64_t e = 0; e < edges; e++) {
        if (u[e] >= *n || v[e] >= *n) {
            set_error("edge " + std::to_string(e) + " has an endpoint >= n = " + std::to_string(*n));
            return CAC_ERR_PARSE;
        }
    }
    return CAC_OK;
}

int cac_graph_load_file(cac_ctx *ctx, const char *path, cac_graph **out) {
    if (!ctx || !path || !out) { set_error("cac_graph_load_file: invalid argument"); return CAC_ERR_INVALID; }
    uint32_t n;
    uint64_t m;
    CAC_TRY(cac_parse_header(path, &n, &m));
    uint32_t *buf = nullptr;
    const size_t bytes = (size_t)(m ? m : 1) * 12;
    if (cudaMallocHost((void **)&buf, bytes) != cudaSuccess) {
        cudaGetLastError();
        set_error("cudaMallocHost failed for the parse buffer");
        return CAC_ERR_OOM;
    }
    uint32_t *u = buf, *v = buf + (m ? m : 1), *w = buf + 2 * (m ? m : 1);
    int st = cac_parse_file(path, &n, &m, u, v, w, m);
    if (st == CAC_OK) st = cac_graph_from_edges(ctx, n, m, u, v, w, CAC_HOST, out);
    if (st == CAC_OK) cudaStreamSynchronize(ctx->stream);
    cudaFreeHost(buf);
    return st;
}

}  // extern "C"
