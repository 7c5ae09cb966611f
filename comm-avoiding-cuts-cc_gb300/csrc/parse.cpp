// Edge-list reader for the reference's input format (src/input/GraphInputIterator.cpp:3-36):
// the first line is skipped unconditionally, then `n m` (unsigned), then m triples `u v w`
// read as unsigned, separated by any whitespace. The reference throws through ifstream
// failbits on malformed input (GraphInputIterator.hpp:19); here the reader returns
// CAC_ERR_IO / CAC_ERR_PARSE with a message instead.
//
// The triples are parsed by all host threads at once: the body is split into chunks at
// whitespace, a first pass counts the tokens of every chunk, and the second pass converts
// each chunk straight into the caller's arrays at its token offset.
//
// Binary cache: a parsed edge list can be written once and read back without parsing. Layout
// (little-endian): "CACG", u32 version (1), u32 n, u32 flags (bit 0: weights stored), u64 m,
// u64 total weight, then u[m], v[m] and, with bit 0, w[m] as u32 (weights 1 otherwise). The
// readers below recognise the magic, so every loader and command line accepts either form.
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
constexpr char kCacheMagic[4] = {'C', 'A', 'C', 'G'};
constexpr uint32_t kCacheVersion = 1;
constexpr size_t kCacheHeader = 32;

struct CacheHeader {
    uint32_t n = 0, flags = 0;
    uint64_t m = 0, total = 0;
};

uint32_t get_u32(const unsigned char *p) {
    return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24;
}
uint64_t get_u64(const unsigned char *p) { return (uint64_t)get_u32(p) | (uint64_t)get_u32(p + 4) << 32; }
void put_u32(unsigned char *p, uint32_t x) {
    for (int i = 0; i < 4; i++) p[i] = (unsigned char)(x >> (8 * i));
}
void put_u64(unsigned char *p, uint64_t x) {
    put_u32(p, (uint32_t)x);
    put_u32(p + 4, (uint32_t)(x >> 32));
}
bool host_little_endian() {
    const uint32_t one = 1;
    unsigned char c;
    std::memcpy(&c, &one, 1);
    return c == 1;
}

// 1: the file is a cache (header read into h), 0: not a cache, <0: error
int read_cache_header(FILE *f, const char *path, CacheHeader &h) {
    unsigned char hd[kCacheHeader];
    const size_t got = std::fread(hd, 1, kCacheHeader, f);
    // the magic and a binary version word: a text file whose (skipped) first line starts with the
    // magic still reads as text
    if (got < 8 || std::memcmp(hd, kCacheMagic, 4) != 0 || get_u32(hd + 4) != kCacheVersion) return 0;
    if (got < kCacheHeader) {
        set_error(std::string("truncated graph cache header in ") + path);
        return CAC_ERR_PARSE;
    }
    h.n = get_u32(hd + 8);
    h.flags = get_u32(hd + 12);
    h.m = get_u64(hd + 16);
    h.total = get_u64(hd + 24);
    return 1;
}

// Reads a cache's arrays (after its header) into the caller's arrays, checks its length, its
// endpoints and its total weight.
int read_cache_body(FILE *f, const char *path, const CacheHeader &h, uint32_t *u, uint32_t *v, uint32_t *w) {
    const uint64_t m = h.m;
    auto read_u32s = [&](uint32_t *dst) -> bool {
        if (m == 0) return true;
        if (std::fread(dst, 4, (size_t)m, f) != (size_t)m) return false;
        if (!host_little_endian())
            for (uint64_t i = 0; i < m; i++) dst[i] = get_u32(reinterpret_cast<const unsigned char *>(dst + i));
        return true;
    };
    std::vector<uint32_t> wtmp;
    uint32_t *wd = w;
    if ((h.flags & 1u) && !wd) {
        wtmp.resize(m ? m : 1);
        wd = wtmp.data();
    }
    if (!read_u32s(u) || !read_u32s(v) || ((h.flags & 1u) && !read_u32s(wd))) {
        set_error(std::string("truncated graph cache ") + path);
        return CAC_ERR_PARSE;
    }
    if (std::fgetc(f) != EOF) {
        set_error(std::string("graph cache ") + path + " is longer than its header declares");
        return CAC_ERR_PARSE;
    }
    if (!(h.flags & 1u) && w)
        for (uint64_t i = 0; i < m; i++) w[i] = 1;
    uint64_t total = 0;
    for (uint64_t e = 0; e < m; e++) {
        if (u[e] >= h.n || v[e] >= h.n) {
            set_error("edge " + std::to_string(e) + " has an endpoint >= n = " + std::to_string(h.n));
            return CAC_ERR_PARSE;
        }
        total += (h.flags & 1u) ? wd[e] : 1u;
    }
    if (total != h.total) {
        set_error(std::string("graph cache ") + path + ": total weight does not match its header");
        return CAC_ERR_PARSE;
    }
    return CAC_OK;
}

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
    {
        CacheHeader h;
        const int c = read_cache_header(f, path, h);
        if (c != 0) {
            std::fclose(f);
            if (c < 0) return c;
            *n = h.n;
            *m = h.m;
            return CAC_OK;
        }
        std::rewind(f);
    }
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
    {
        FILE *f = std::fopen(path, "rb");
        if (!f) { set_error(std::string("cannot open ") + path); return CAC_ERR_IO; }
        CacheHeader h;
        const int c = read_cache_header(f, path, h);
        if (c != 0) {
            int st = c < 0 ? c : CAC_OK;
            if (st == CAC_OK) {
                *n = h.n;
                *m = h.m;
                if (h.m > capacity || (h.m && (!u || !v))) {
                    set_error("cac_parse_file: output capacity " + std::to_string(capacity) + " < edge count " +
                              std::to_string(h.m));
                    st = CAC_ERR_INVALID;
                } else {
                    st = read_cache_body(f, path, h, u, v, w);
                }
            }
            std::fclose(f);
            return st;
        }
        std::fclose(f);
    }
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

int cac_cache_write(const char *path, uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w) {
    if (!path || (m && (!u || !v))) { set_error("cac_cache_write: invalid argument"); return CAC_ERR_INVALID; }
    uint64_t total = 0;
    for (uint64_t e = 0; e < m; e++) {
        if (u[e] >= n || v[e] >= n) {
            set_error("cac_cache_write: edge " + std::to_string(e) + " has an endpoint >= n = " + std::to_string(n));
            return CAC_ERR_INVALID;
        }
        total += w ? w[e] : 1u;
    }
    unsigned char hd[kCacheHeader] = {};
    std::memcpy(hd, kCacheMagic, 4);
    put_u32(hd + 4, kCacheVersion);
    put_u32(hd + 8, n);
    put_u32(hd + 12, w ? 1u : 0u);
    put_u64(hd + 16, m);
    put_u64(hd + 24, total);
    FILE *f = std::fopen(path, "wb");
    if (!f) { set_error(std::string("cannot create ") + path); return CAC_ERR_IO; }
    bool ok = std::fwrite(hd, 1, kCacheHeader, f) == kCacheHeader;
    auto write_u32s = [&](const uint32_t *src) {
        if (!ok || m == 0) return;
        if (host_little_endian()) {
            ok = std::fwrite(src, 4, (size_t)m, f) == (size_t)m;
            return;
        }
        std::vector<unsigned char> tmp(4 * (size_t)std::min<uint64_t>(m, 1 << 20));
        for (uint64_t e0 = 0; e0 < m && ok; e0 += tmp.size() / 4) {
            const uint64_t k = std::min<uint64_t>(m - e0, tmp.size() / 4);
            for (uint64_t i = 0; i < k; i++) put_u32(tmp.data() + 4 * i, src[e0 + i]);
            ok = std::fwrite(tmp.data(), 4, (size_t)k, f) == (size_t)k;
        }
    };
    write_u32s(u);
    write_u32s(v);
    if (w) write_u32s(w);
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) { set_error(std::string("writing ") + path + " failed"); return CAC_ERR_IO; }
    return CAC_OK;
}

int cac_cache_convert(const char *input_path, const char *cache_path) {
    if (!input_path || !cache_path) { set_error("cac_cache_convert: invalid argument"); return CAC_ERR_INVALID; }
    uint32_t n;
    uint64_t m;
    CAC_TRY(cac_parse_header(input_path, &n, &m));
    std::vector<uint32_t> u(m ? m : 1), v(m ? m : 1), w(m ? m : 1);
    CAC_TRY(cac_parse_file(input_path, &n, &m, u.data(), v.data(), w.data(), m));
    return cac_cache_write(cache_path, n, m, u.data(), v.data(), w.data());
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
