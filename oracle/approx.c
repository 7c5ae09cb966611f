/*
 * ORACLE (test infrastructure) — approx_cut (src/ApproximateCut.cpp:10-87).
 *
 * The reference sums the edge weights w, and for levels i = 1..ceil(ln w) keeps every edge of
 * each of `trials` copies iff Binomial(weight, 2^-i) > 0, runs CC over the disjoint union of the
 * copies and stops at the first level with more than `trials` components; the answer is 2^i
 * (2^0 when no level disconnects). trials = ceil(ln(1-p) / ln(1-e^-0.75)) (:82-87).
 *
 * libcac's counter-addressed keep test (the reference draws through libstdc++'s
 * binomial_distribution): P(Binomial(w, q) > 0) = 1 - (1-q)^w, so edge e of copy j at level i
 * is kept iff x >= F(i, w_e), where x is draw e_local of the stream with key
 * (seed + r, i, j, 1) (r = the virtual rank owning the edge's slice, e_local its index in the
 * slice, round 0) and F(i, w) is (1 - 2^-i)^w in 0.64 fixed point, evaluated by square-and-
 * multiply with truncating 64x64->128-bit products. Integer-only, so host and device agree bit
 * for bit. Zero-weight edges are never kept.
 */
#include <stdlib.h>
#include <math.h>
#include "oracle.h"

static uint64_t mulhi64(uint64_t a, uint64_t b) { return (uint64_t)(((unsigned __int128)a * b) >> 64); }

uint32_t orc_approx_trials(double p) {
    double alpha = log(1 - exp(-(double)0.75));
    return (uint32_t)ceil(log((double)1.0 - p) / alpha);
}

uint64_t orc_keep_threshold(uint32_t level, uint32_t w) {
    uint64_t base = 0 - (1ull << (64 - level)); /* 1 - 2^-level */
    uint64_t res = base, b = base;
    uint32_t e = w - 1;
    while (e) {
        if (e & 1) res = mulhi64(res, b);
        b = mulhi64(b, b);
        e >>= 1;
    }
    return res;
}

static uint32_t afind(uint32_t *p, uint32_t x) { while (p[x] != x) { p[x] = p[p[x]]; x = p[x]; } return x; }

uint64_t orc_approx_cut(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w,
                        double success_probability, uint32_t seed, uint32_t ranks, uint32_t *levels_out) {
    if (ranks == 0) ranks = 1;
    uint64_t total = 0;
    for (uint64_t e = 0; e < m; e++) total += w[e];
    uint32_t iterations = (uint32_t)ceil(log((double)total));
    uint32_t trials = orc_approx_trials(success_probability);
    uint64_t nv = (uint64_t)n * trials;
    uint32_t *p = (uint32_t *)malloc(sizeof(uint32_t) * (nv ? nv : 1));
    uint64_t portion = m / ranks;
    uint32_t first = 0;
    for (uint32_t i = 1; i <= iterations && i <= 63; i++) {
        for (uint64_t x = 0; x < nv; x++) p[x] = (uint32_t)x;
        uint64_t comps = nv;
        for (uint32_t j = 0; j < trials; j++) {
            for (uint32_t r = 0; r < ranks; r++) {
                uint64_t from = portion * r, to = (r == ranks - 1) ? m : portion * (r + 1);
                uint64_t key[4] = {(uint32_t)(seed + r), i, j, 1};
                for (uint64_t e = from; e < to; e++) {
                    if (w[e] == 0) continue;
                    uint64_t x = orc_draw64(key, 0, e - from);
                    if (x < orc_keep_threshold(i, w[e])) continue;
                    uint32_t a = afind(p, u[e] + j * n), b = afind(p, v[e] + j * n);
                    if (a != b) { if (a < b) p[b] = a; else p[a] = b; comps--; }
                }
            }
        }
        if (comps > trials) { first = i; break; }
    }
    free(p);
    if (levels_out) *levels_out = first;
    return (uint64_t)1 << first;
}
