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
 *
 * Level count: the reference takes ceil(ln w) of the weight sum of the calling rank's own slice
 * (`w` at :19-30 is the local sum; the reduced `weightUpperBound` is never used). All ranks run
 * the same collectives level by level, so the run is well defined only while every rank is still
 * in its loop; both restatements here run min over ranks of ceil(ln w_r) levels (a rank whose
 * slice weighs 0 runs none), which gives the reference's answer wherever it has one.
 *
 * orc_approx_cut_stream replays the reference's own draws instead: rank r's engine
 * sitmo::prng_engine(seed + r) (ApproximateCut.hpp:35, .cpp:33) is consumed in the reference's
 * order (level, copy, slice edge), one std::binomial_distribution<int>(w, 2^-i) per edge, plus
 * one raw output per level for the CC seed (:50-58). The distribution lives in libstdc++
 * (third-party; GCC 13 here), restated from its published algorithm:
 *   - std::generate_canonical<double, 53> on a 32-bit engine takes two outputs x0, x1 and returns
 *     (x0 + x1 * 2^32) / 2^64 in double arithmetic, clamped below 1;
 *   - binomial_distribution(t, p), p <= 1/2, with t * p < 8: the waiting-time method (Devroye,
 *     Non-Uniform Random Variate Generation, 1986, ch. X.4): add E_k / (t - k), E_k = -ln(1 - U_k),
 *     for k = 0, 1, ... until the sum exceeds q = -ln(1 - p) or k reaches t; the result is the
 *     number of terms added minus one (t when k reached t). A draw with t = 0 takes no output.
 * Draws outside t * p < 8 (libstdc++ switches to a rejection method there) are not restated:
 * the function then returns 0. Pinned against oracle/refbuild's binom_stream harness and the
 * reference's approx_cut executable (tests/golden/approx_stream.json).
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

/* ceil(ln w) as the reference's `(unsigned) std::ceil(std::log(w))` (:30) */
static uint32_t level_count(uint64_t w) { return w ? (uint32_t)ceil(log((double)w)) : 0; }

/* min over ranks of the level count of the rank's slice (slices as GraphInputIterator::loadSlice,
 * src/input/GraphInputIterator.hpp:77-93: rank r < P-1 owns [r*floor(m/P), (r+1)*floor(m/P)), the
 * last rank the rest) */
static uint32_t slice_levels(uint64_t m, const uint32_t *w, uint32_t ranks) {
    uint64_t portion = m / ranks;
    uint32_t best = UINT32_MAX;
    for (uint32_t r = 0; r < ranks; r++) {
        uint64_t from = portion * r, to = (r == ranks - 1) ? m : portion * (r + 1), sum = 0;
        for (uint64_t e = from; e < to; e++) sum += w[e];
        uint32_t l = level_count(sum);
        if (l < best) best = l;
    }
    return best;
}

/* the reference engine sitmo::prng_engine(seed), read output by output (lib/prng_engine.hpp:195-212) */
typedef struct {
    uint64_t key[4], k, blk, out[4];
} ref_engine;

static void ref_engine_init(ref_engine *s, uint32_t seed) {
    s->key[0] = seed; s->key[1] = s->key[2] = s->key[3] = 0;
    s->k = 0;
    s->blk = UINT64_MAX;
}

static uint32_t ref_engine_next(ref_engine *s) {
    uint64_t b = s->k >> 3;
    if (b != s->blk) {
        uint64_t ctr[4] = {b, 0, 0, 0};
        orc_sitmo_block(s->key, ctr, s->out);
        s->blk = b;
    }
    unsigned idx = (unsigned)(s->k & 7);
    s->k++;
    return (uint32_t)(s->out[idx >> 1] >> (32 * (idx & 1)));
}

/* std::generate_canonical<double, 53> on the 32-bit engine */
static double ref_canonical(ref_engine *s) {
    double sum = (double)ref_engine_next(s);
    sum += (double)ref_engine_next(s) * 4294967296.0;
    double u = sum / 18446744073709551616.0;
    if (u >= 1.0) u = nextafter(1.0, 0.0);
    return u;
}

/* std::binomial_distribution<int>(t, p) for p <= 1/2 and t * p < 8 (waiting-time method);
 * q = -ln(1 - p) */
static int ref_binomial_waiting(ref_engine *s, int t, double q) {
    int x = 0;
    double sum = 0.0;
    do {
        if (t == x) return x;
        double e = -log(1.0 - ref_canonical(s));
        sum += e / (t - x);
        x += 1;
    } while (sum <= q);
    return x - 1;
}

int orc_ref_binomial_draws(uint32_t seed, uint32_t level, uint64_t count, const uint32_t *w, uint32_t nw,
                           int32_t *draws, uint32_t *next_output) {
    ref_engine s;
    ref_engine_init(&s, seed);
    double p = pow(2, -(int)level), q = -log(1 - p);
    for (uint64_t k = 0; k < count; k++) {
        int t = (int)w[k % nw];
        if (t * p >= 8) return -1;
        draws[k] = ref_binomial_waiting(&s, t, q);
    }
    *next_output = ref_engine_next(&s);
    return 0;
}

uint64_t orc_approx_cut_stream(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w,
                               double success_probability, uint32_t seed, uint32_t ranks, uint32_t *levels_out) {
    if (ranks == 0) ranks = 1;
    uint32_t iterations = slice_levels(m, w, ranks);
    uint32_t trials = orc_approx_trials(success_probability);
    uint64_t nv = (uint64_t)n * trials;
    uint32_t *p = (uint32_t *)malloc(sizeof(uint32_t) * (nv ? nv : 1));
    ref_engine *eng = (ref_engine *)malloc(sizeof(ref_engine) * ranks);
    for (uint32_t r = 0; r < ranks; r++) ref_engine_init(&eng[r], seed + r);
    uint64_t portion = m / ranks;
    uint32_t first = 0;
    uint64_t result = 0;
    for (uint32_t i = 1; i <= iterations && i <= 63; i++) {
        double pi = pow(2, -(int)i), q = -log(1 - pi);
        for (uint64_t x = 0; x < nv; x++) p[x] = (uint32_t)x;
        uint64_t comps = nv;
        for (uint32_t r = 0; r < ranks; r++) {
            uint64_t from = portion * r, to = (r == ranks - 1) ? m : portion * (r + 1);
            for (uint32_t j = 0; j < trials; j++) {
                for (uint64_t e = from; e < to; e++) {
                    int t = (int)w[e];
                    if (t * pi >= 8) goto unsupported;
                    if (ref_binomial_waiting(&eng[r], t, q) <= 0) continue;
                    uint32_t a = afind(p, u[e] + j * n), b = afind(p, v[e] + j * n);
                    if (a != b) { if (a < b) p[b] = a; else p[a] = b; comps--; }
                }
            }
            ref_engine_next(&eng[r]); /* the seed of this level's CC */
        }
        if (comps > trials) { first = i; break; }
    }
    result = (uint64_t)1 << first;
    if (levels_out) *levels_out = first;
unsupported:
    free(eng);
    free(p);
    return result;
}

uint64_t orc_approx_cut(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w,
                        double success_probability, uint32_t seed, uint32_t ranks, uint32_t *levels_out) {
    if (ranks == 0) ranks = 1;
    uint32_t iterations = slice_levels(m, w, ranks);
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
