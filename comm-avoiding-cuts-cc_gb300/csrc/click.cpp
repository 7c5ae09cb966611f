// CLICK: the reference's in-memory test graph (src/input/CLICK.hpp:10-49), as approx_cut loads it on
// P ranks (ApproximateCut.hpp:35 seeds rank r with seed + r; :70-82 calls the generator).
//
// The complete graph on n vertices, edges (i, j), i < j, enumerated row by row. Rank r owns the
// enumeration range [r * floor(E / P), (r + 1) * floor(E / P)), E = n (n - 1) / 2; the remaining
// E mod P edges belong to no rank (the reference's last-rank test, rank == group_size, never
// holds), so the graph has P * floor(E / P) edges. Rank r draws its weights in enumeration order
// from one std::mt19937 seeded with seed + r: a pair in the same cluster (i mod 10 == j mod 10)
// takes max(0, N(8, 4)) from one std::normal_distribution<float>, any other pair max(0, N(4, 4))
// from a second one, truncated to an integer. The draws come from the C++ standard library, as in
// the reference, so the graph is the reference's edge for edge; the ranks are generated on
// separate host threads.
#include <algorithm>
#include <random>
#include <thread>
#include <vector>

#include "cac_internal.h"

namespace cac {
namespace {

constexpr uint32_t kClusters = 10;

// first pair (i, j) of enumeration position pos among the pairs i < j of n vertices
void pair_at(uint64_t n, uint64_t pos, uint32_t &i, uint32_t &j) {
    uint64_t lo = 0, hi = n - 2;  // last row whose first position <= pos
    auto start = [&](uint64_t r) { return r * (n - 1) - r * (r - 1) / 2; };
    while (lo < hi) {
        const uint64_t mid = (lo + hi + 1) / 2;
        if (start(mid) <= pos) lo = mid; else hi = mid - 1;
    }
    i = (uint32_t)lo;
    j = (uint32_t)(lo + 1 + (pos - start(lo)));
}

void click_slice(uint32_t n, uint64_t from, uint64_t to, uint32_t seed, uint32_t *u, uint32_t *v, uint32_t *w) {
    std::mt19937 gen(seed);
    std::normal_distribution<float> mates(8, 4);
    std::normal_distribution<float> non_mates(4, 4);
    if (from >= to) return;
    uint32_t i, j;
    pair_at(n, from, i, j);
    for (uint64_t e = 0; e < to - from; e++) {
        const float x = (i % kClusters == j % kClusters) ? mates(gen) : non_mates(gen);
        u[e] = i;
        v[e] = j;
        w[e] = (uint32_t)(unsigned long)std::max(0.f, x);
        if (++j == n) {
            i++;
            j = i + 1;
        }
    }
}

}  // namespace

int click_edges(uint32_t n, uint32_t ranks, uint32_t seed, uint32_t *u, uint32_t *v, uint32_t *w, uint64_t capacity,
                uint64_t *m_out) {
    if (ranks == 0) ranks = 1;
    if (n < 2 || (uint64_t)n * (n - 1) / 2 > 0xFFFFFFFFull) {
        set_error("CLICK: the vertex count must be at least 2 and give at most 2^32 - 1 edges");
        return CAC_ERR_INVALID;
    }
    const uint64_t E = (uint64_t)n * (n - 1) / 2;
    const uint64_t portion = E / ranks;
    const uint64_t m = portion * ranks;
    if (m_out) *m_out = m;
    if (!u) return CAC_OK;  // size query
    if (!v || !w || capacity < m) {
        set_error("CLICK: output arrays missing or smaller than the " + std::to_string(m) + " edges");
        return CAC_ERR_INVALID;
    }
    const uint32_t hw = std::max(1u, std::thread::hardware_concurrency());
    for (uint32_t r0 = 0; r0 < ranks; r0 += hw) {
        std::vector<std::thread> pool;
        for (uint32_t r = r0; r < std::min(ranks, r0 + hw); r++) {
            const uint64_t from = portion * r;
            pool.emplace_back(click_slice, n, from, from + portion, seed + r, u + from, v + from, w + from);
        }
        for (auto &t : pool) t.join();
    }
    return CAC_OK;
}

}  // namespace cac

using namespace cac;

extern "C" {

int cac_click_edges(uint32_t n, uint32_t virtual_ranks, uint32_t seed, uint32_t *u, uint32_t *v, uint32_t *w,
                    uint64_t capacity, uint64_t *m) {
    return click_edges(n, virtual_ranks, seed, u, v, w, capacity, m);
}

int cac_graph_click(cac_ctx *ctx, uint32_t n, uint32_t virtual_ranks, uint32_t seed, cac_graph **out) {
    if (!ctx || !out) {
        set_error("cac_graph_click: invalid argument");
        return CAC_ERR_INVALID;
    }
    uint64_t m = 0;
    CAC_TRY(click_edges(n, virtual_ranks, seed, nullptr, nullptr, nullptr, 0, &m));
    std::vector<uint32_t> u(m), v(m), w(m);
    CAC_TRY(click_edges(n, virtual_ranks, seed, u.data(), v.data(), w.data(), m, &m));
    return cac_graph_from_edges(ctx, n, m, u.data(), v.data(), w.data(), CAC_HOST, out);
}

}  // extern "C"
