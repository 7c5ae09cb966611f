/*
 * ORACLE (test infrastructure) — minimum cut.
 *
 * 1. Exact cut: Stoer-Wagner maximum-adjacency search, the algorithm of the reference's base
 *    case (src/karger-stein/co_mincut_base_case.hpp:52-144, deterministic_cut_sparse), on a
 *    dense matrix (small n) or on edge lists with a binary heap and merged vertex sets
 *    (larger n). The min-cut VALUE is unique, so any correct exact method is a valid oracle.
 *
 * 2. Trial budget: SquareRootCut::intermediate_size / numberOfTrials (SquareRootCut.cpp:63-83)
 *    and comincut::target_number_of_vertices_for_contraction / min_success_in_one_trial
 *    (co_mincut.cpp:18-41), restated with the same double-precision expressions.
 *
 * 3. Replay of one counter-addressed square_root trial. The structure follows the reference:
 *      Stage 1  iterated sampling to t = min(n, ceil(2 sqrt(m) + 1)) vertices
 *               (SequentialSquareRootCut.cpp:21-67): rounds of (current vertex count) draws,
 *               each edge drawn with probability proportional to its weight among the edges
 *               that are not loops at the start of the round, contracted in draw order until
 *               exactly t vertices remain;
 *      Stage 2  compact to a dense t x t matrix (AdjacencyListGraph::compact + as_dense_graph);
 *      Stage 3  Karger-Stein recursion (co_mincut.h:176-223): fan-out 2, each child contracts a
 *               copy to max(ceil(n/sqrt 2)+1, 128) vertices by weighted random contraction,
 *               base case n <= 128 solved exactly (co_mincut_base_case.hpp:164-221); the trial
 *               value is min(minimum weighted degree, every leaf's exact cut).
 *    What is libcac's own definition (the reference draws through libstdc++'s
 *    uniform_int_distribution and sum_tree, whose consumption is data dependent):
 *      - draw d of round rho of a stream with key K is the u64 word d%4 of the sitmo block at
 *        counter (d/4, rho, 0, 0); trial (r, i) uses key (seed + r, i, tag, 0) with tag 1 for
 *        Stage 1 and tag 1 + h for the Karger-Stein child with heap index h (root h = 1,
 *        children 2h, 2h + 1);
 *      - a draw x selects over total weight W by y = floor(x * W / 2^64) and takes the first
 *        element (edge-array order in Stage 1, row-major matrix order in Stage 3) whose
 *        inclusive weight prefix exceeds y;
 *      - contracted vertices are renamed to the rank of their smallest member;
 *      - a Karger-Stein child that has not reached its target after (current vertex count)
 *        draws replaces its matrix by the quotient and draws a fresh round (round rho + 1).
 *    The heavy-edge PR passes of the reference change no returned value (they only contract
 *    edges at least as heavy as the current upper bound) and are not part of this definition.
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "oracle.h"

#define U64MAX 0xFFFFFFFFFFFFFFFFull

static uint64_t mulhi64(uint64_t a, uint64_t b) { return (uint64_t)(((unsigned __int128)a * b) >> 64); }

/* ------------------------------------------------------------------ exact cut */

uint64_t orc_stoer_wagner_dense(uint32_t n, uint64_t *mat) {
    if (n < 2) return U64MAX;
    uint32_t *act = (uint32_t *)malloc(sizeof(uint32_t) * n);
    uint64_t *key = (uint64_t *)malloc(sizeof(uint64_t) * n);
    uint8_t *in_a = (uint8_t *)malloc(n);
    for (uint32_t i = 0; i < n; i++) act[i] = i;
    uint32_t cnt = n;
    uint64_t best = U64MAX;
    while (cnt > 1) {
        for (uint32_t i = 0; i < cnt; i++) { key[act[i]] = 0; in_a[act[i]] = 0; }
        uint32_t prev = act[0], last = act[0];
        for (uint32_t step = 0; step < cnt; step++) {
            uint32_t s = n;
            uint64_t bk = 0;
            for (uint32_t i = 0; i < cnt; i++) {
                uint32_t x = act[i];
                if (!in_a[x] && (s == n || key[x] > bk)) { s = x; bk = key[x]; }
            }
            in_a[s] = 1;
            if (step + 1 == cnt) { last = s; break; }
            prev = s;
            const uint64_t *row = mat + (size_t)s * n;
            for (uint32_t i = 0; i < cnt; i++) {
                uint32_t x = act[i];
                if (!in_a[x]) key[x] += row[x];
            }
        }
        if (key[last] < best) best = key[last];
        /* merge `last` into `prev` */
        uint64_t *rp = mat + (size_t)prev * n, *rl = mat + (size_t)last * n;
        for (uint32_t i = 0; i < cnt; i++) {
            uint32_t x = act[i];
            rp[x] += rl[x];
            mat[(size_t)x * n + prev] = rp[x];
        }
        rp[prev] = 0;
        for (uint32_t i = 0; i < cnt; i++)
            if (act[i] == last) { act[i] = act[cnt - 1]; break; }
        cnt--;
        /* keep the active list ordered so that ties resolve to the lowest index */
        for (uint32_t i = 1; i < cnt; i++) {
            uint32_t x = act[i], j = i;
            while (j > 0 && act[j - 1] > x) { act[j] = act[j - 1]; j--; }
            act[j] = x;
        }
    }
    free(act); free(key); free(in_a);
    return best;
}

/* heap-based Stoer-Wagner over edge lists; vertex sets merged through a union-find */
typedef struct { uint64_t k; uint32_t v; } hnode;
static void hpush(hnode *h, size_t *sz, uint64_t k, uint32_t v) {
    size_t i = (*sz)++;
    while (i > 0) {
        size_t p = (i - 1) / 2;
        if (h[p].k >= k) break;
        h[i] = h[p]; i = p;
    }
    h[i].k = k; h[i].v = v;
}
static hnode hpop(hnode *h, size_t *sz) {
    hnode top = h[0], x = h[--(*sz)];
    size_t i = 0;
    for (;;) {
        size_t c = 2 * i + 1;
        if (c >= *sz) break;
        if (c + 1 < *sz && h[c + 1].k > h[c].k) c++;
        if (h[c].k <= x.k) break;
        h[i] = h[c]; i = c;
    }
    if (*sz) h[i] = x;
    return top;
}
static uint32_t sfind(uint32_t *p, uint32_t x) { while (p[x] != x) { p[x] = p[p[x]]; x = p[x]; } return x; }

static uint64_t sw_sparse(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w) {
    /* CSR of the original graph (both directions) */
    uint64_t *off = (uint64_t *)calloc(n + 1, sizeof(uint64_t));
    for (uint64_t e = 0; e < m; e++) if (u[e] != v[e]) { off[u[e] + 1]++; off[v[e] + 1]++; }
    for (uint32_t i = 0; i < n; i++) off[i + 1] += off[i];
    uint32_t *adj = (uint32_t *)malloc(sizeof(uint32_t) * (off[n] ? off[n] : 1));
    uint64_t *aw = (uint64_t *)malloc(sizeof(uint64_t) * (off[n] ? off[n] : 1));
    uint64_t *fill = (uint64_t *)malloc(sizeof(uint64_t) * (n + 1));
    memcpy(fill, off, sizeof(uint64_t) * (n + 1));
    for (uint64_t e = 0; e < m; e++) {
        if (u[e] == v[e]) continue;
        adj[fill[u[e]]] = v[e]; aw[fill[u[e]]++] = w[e];
        adj[fill[v[e]]] = u[e]; aw[fill[v[e]]++] = w[e];
    }
    /* members of each super-vertex as linked lists */
    uint32_t *p = (uint32_t *)malloc(sizeof(uint32_t) * n), *next = (uint32_t *)malloc(sizeof(uint32_t) * n);
    uint32_t *tail = (uint32_t *)malloc(sizeof(uint32_t) * n);
    for (uint32_t i = 0; i < n; i++) { p[i] = i; next[i] = U64MAX & 0xFFFFFFFFu; tail[i] = i; }
    uint64_t *key = (uint64_t *)malloc(sizeof(uint64_t) * n);
    uint32_t *stamp = (uint32_t *)calloc(n, sizeof(uint32_t));
    uint8_t *done = (uint8_t *)malloc(n);
    hnode *heap = (hnode *)malloc(sizeof(hnode) * (off[n] + n + 1));
    uint64_t best = U64MAX;
    uint32_t cnt = n;
    uint32_t phase = 0;
    while (cnt > 1) {
        phase++;
        size_t hs = 0;
        uint32_t start = U64MAX & 0xFFFFFFFFu;
        for (uint32_t i = 0; i < n; i++) if (p[i] == i) { key[i] = 0; done[i] = 0; stamp[i] = phase; if (start > i) start = i; }
        hpush(heap, &hs, 0, start);
        uint32_t prev = start, last = start, added = 0;
        while (hs > 0) {
            hnode t = hpop(heap, &hs);
            uint32_t s = t.v;
            if (done[s] || t.k != key[s]) continue;
            done[s] = 1;
            added++;
            if (added == cnt) { last = s; break; }
            prev = s;
            for (uint32_t x = s; x != (U64MAX & 0xFFFFFFFFu); x = next[x]) {
                for (uint64_t k = off[x]; k < off[x + 1]; k++) {
                    uint32_t y = sfind(p, adj[k]);
                    if (y == s || done[y]) continue;
                    key[y] += aw[k];
                    hpush(heap, &hs, key[y], y);
                }
            }
        }
        if (added < cnt) { best = 0; break; } /* disconnected */
        if (key[last] < best) best = key[last];
        /* merge last into prev */
        p[last] = prev;
        next[tail[prev]] = last;
        tail[prev] = tail[last];
        cnt--;
    }
    free(off); free(adj); free(aw); free(fill); free(p); free(next); free(tail);
    free(key); free(stamp); free(done); free(heap);
    return best;
}

/* Nagamochi-Ono-Ibaraki exact minimum cut (H. Nagamochi, T. Ono, T. Ibaraki, "Implementing an
 * efficient minimum capacity cut algorithm", Math. Programming 67, 1994) for graphs too large for
 * one Stoer-Wagner phase per vertex. Each phase runs one maximum-adjacency ordering of the
 * current (merged, loop-free) graph from vertex 0; when vertex x is scanned, every unscanned
 * neighbour y gets r(y) += w(x, y) and the edge is given q = r(y). The maximum-adjacency lemma
 * gives q <= lambda(x, y), the local edge connectivity of its ends, so every edge with
 * q >= best (best = the smallest cut found so far, starting at the minimum weighted degree) can
 * be contracted without losing a cut below best. The last two vertices of the ordering are
 * merged too (Stoer-Wagner's lemma: lambda of that pair is r(last) = d(last) >= best), so every
 * phase removes at least one vertex. After contracting, best takes the new minimum weighted
 * degree. A vertex left unscanned when the heap empties means the graph is disconnected: 0.
 * The value is the same as the Stoer-Wagner routines above (checked by the oracle pin tests). */
typedef struct { uint64_t key; uint64_t w; } kedge;
static int kedge_cmp(const void *a, const void *b) {
    const uint64_t x = ((const kedge *)a)->key, y = ((const kedge *)b)->key;
    return x < y ? -1 : x > y;
}
uint64_t orc_exact_mincut_noi(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w) {
    if (n < 2) return U64MAX;
    kedge *E = (kedge *)malloc(sizeof(kedge) * (m ? m : 1));
    uint64_t me = 0;
    for (uint64_t e = 0; e < m; e++) {
        if (u[e] == v[e] || w[e] == 0) continue;
        uint32_t a = u[e] < v[e] ? u[e] : v[e], b = u[e] ^ v[e] ^ a;
        E[me].key = ((uint64_t)a << 32) | b; E[me].w = w[e]; me++;
    }
    uint32_t k = n;
    uint64_t best = U64MAX;
    uint64_t *off = (uint64_t *)malloc(sizeof(uint64_t) * (n + 1));
    uint32_t *adj = (uint32_t *)malloc(sizeof(uint32_t) * (2 * me + 1));
    uint64_t *aw = (uint64_t *)malloc(sizeof(uint64_t) * (2 * me + 1));
    uint64_t *fill = (uint64_t *)malloc(sizeof(uint64_t) * (n + 1));
    uint64_t *r = (uint64_t *)malloc(sizeof(uint64_t) * n), *deg = (uint64_t *)malloc(sizeof(uint64_t) * n);
    uint8_t *done = (uint8_t *)malloc(n);
    uint32_t *p = (uint32_t *)malloc(sizeof(uint32_t) * n), *lab = (uint32_t *)malloc(sizeof(uint32_t) * n);
    hnode *heap = (hnode *)malloc(sizeof(hnode) * (2 * me + n + 1));
    for (;;) {
        /* merge parallel edges: sort by (min, max) end and sum */
        qsort(E, me, sizeof(kedge), kedge_cmp);
        uint64_t j = 0;
        for (uint64_t e = 0; e < me; e++) {
            if (j && E[j - 1].key == E[e].key) E[j - 1].w += E[e].w;
            else E[j++] = E[e];
        }
        me = j;
        memset(deg, 0, sizeof(uint64_t) * k);
        for (uint64_t e = 0; e < me; e++) { deg[E[e].key >> 32] += E[e].w; deg[(uint32_t)E[e].key] += E[e].w; }
        for (uint32_t i = 0; i < k; i++) if (deg[i] < best) best = deg[i];
        if (k <= 2 || best == 0) break;
        /* CSR, both directions */
        memset(off, 0, sizeof(uint64_t) * (k + 1));
        for (uint64_t e = 0; e < me; e++) { off[(E[e].key >> 32) + 1]++; off[(uint32_t)E[e].key + 1]++; }
        for (uint32_t i = 0; i < k; i++) off[i + 1] += off[i];
        memcpy(fill, off, sizeof(uint64_t) * (k + 1));
        for (uint64_t e = 0; e < me; e++) {
            const uint32_t a = (uint32_t)(E[e].key >> 32), b = (uint32_t)E[e].key;
            adj[fill[a]] = b; aw[fill[a]++] = E[e].w;
            adj[fill[b]] = a; aw[fill[b]++] = E[e].w;
        }
        /* one maximum-adjacency ordering; contractible pairs joined in a union-find */
        for (uint32_t i = 0; i < k; i++) { r[i] = 0; done[i] = 0; p[i] = i; }
        size_t hs = 0;
        hpush(heap, &hs, 0, 0);
        uint32_t scanned = 0, prev = 0, last = 0;
        while (hs > 0) {
            hnode t = hpop(heap, &hs);
            const uint32_t x = t.v;
            if (done[x] || t.k != r[x]) continue;
            done[x] = 1;
            scanned++;
            prev = last; last = x;
            for (uint64_t q = off[x]; q < off[x + 1]; q++) {
                const uint32_t y = adj[q];
                if (done[y]) continue;
                r[y] += aw[q];
                if (r[y] >= best) { uint32_t a = sfind(p, x), b = sfind(p, y); if (a != b) p[a < b ? b : a] = a < b ? a : b; }
                hpush(heap, &hs, r[y], y);
            }
        }
        if (scanned < k) { best = 0; break; }
        { uint32_t a = sfind(p, prev), b = sfind(p, last); if (a != b) p[a < b ? b : a] = a < b ? a : b; }
        /* contract: label = rank of each set's smallest member */
        uint32_t nk = 0;
        for (uint32_t i = 0; i < k; i++) { const uint32_t rt = sfind(p, i); lab[i] = rt == i ? nk++ : lab[rt]; }
        j = 0;
        for (uint64_t e = 0; e < me; e++) {
            const uint32_t a = lab[E[e].key >> 32], b = lab[(uint32_t)E[e].key];
            if (a == b) continue;
            E[j].key = a < b ? ((uint64_t)a << 32) | b : ((uint64_t)b << 32) | a;
            E[j].w = E[e].w; j++;
        }
        me = j;
        k = nk;
        if (k < 2) break;
    }
    free(E); free(off); free(adj); free(aw); free(fill); free(r); free(deg); free(done); free(p); free(lab);
    free(heap);
    return best;
}

uint64_t orc_exact_mincut(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w) {
    if (n < 2) return U64MAX;
    if (n <= 1024) {
        uint64_t *mat = (uint64_t *)calloc((size_t)n * n, sizeof(uint64_t));
        for (uint64_t e = 0; e < m; e++) {
            if (u[e] == v[e]) continue;
            mat[(size_t)u[e] * n + v[e]] += w[e];
            mat[(size_t)v[e] * n + u[e]] += w[e];
        }
        uint64_t r = orc_stoer_wagner_dense(n, mat);
        free(mat);
        return r;
    }
    return sw_sparse(n, m, u, v, w);
}

/* ------------------------------------------------------------------ trial budget */

int orc_ks_target(int n) {
    int t = (int)ceil((double)n / sqrt((double)2)) + 1;
    return t > 128 ? t : 128;
}

double orc_min_success_in_one_trial(int n) {
    if (n <= 128) return 1;
    double r = orc_min_success_in_one_trial(orc_ks_target(n));
    return 1.0 - pow((1 - 0.5 * r), 2);
}

uint32_t orc_intermediate_size(uint32_t n, uint64_t m) {
    uint32_t c = (uint32_t)ceil(2.0 * sqrt((double)m) + 1);
    return c > n ? n : c;
}

uint32_t orc_number_of_trials(uint32_t n, uint64_t m, double p) {
    double pk = orc_min_success_in_one_trial((int)orc_intermediate_size(n, m));
    double c = 1.0 / (1 - p);
    return (uint32_t)ceil(((double)n * ((double)n * log(c))) / (2.0 * 2.0 * ((double)m * pk)));
}

/* ------------------------------------------------------------------ trial replay */

static uint32_t qfind(uint32_t *p, uint32_t x) { while (p[x] != x) { p[x] = p[p[x]]; x = p[x]; } return x; }

/* rank-of-minimum relabel of a union-find over [0, n): lab[v] in [0, k), returns k */
static uint32_t rank_labels(uint32_t n, uint32_t *p, uint32_t *lab) {
    uint32_t *first = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    for (uint32_t i = 0; i < n; i++) first[i] = 0xFFFFFFFFu;
    uint32_t k = 0;
    for (uint32_t i = 0; i < n; i++) {
        uint32_t r = qfind(p, i);
        if (first[r] == 0xFFFFFFFFu) first[r] = k++;
        lab[i] = first[r];
    }
    free(first);
    return k;
}

/* quotient of an n x n matrix by labels in [0, k) */
static uint64_t *quotient(uint32_t n, const uint64_t *g, const uint32_t *lab, uint32_t k) {
    uint64_t *q = (uint64_t *)calloc((size_t)k * k, sizeof(uint64_t));
    for (uint32_t a = 0; a < n; a++) {
        const uint64_t *row = g + (size_t)a * n;
        uint64_t *qrow = q + (size_t)lab[a] * k;
        for (uint32_t b = 0; b < n; b++)
            if (lab[a] != lab[b]) qrow[lab[b]] += row[b];
    }
    return q;
}

/* Contract a dense graph to `target` vertices (see header comment). Returns the new matrix,
 * *n_out its dimension. */
static uint64_t *ks_shrink(uint32_t n, const uint64_t *g0, uint32_t target, const uint64_t key[4], uint32_t *n_out) {
    uint32_t dim = n;
    uint64_t *g = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n * n);
    memcpy(g, g0, sizeof(uint64_t) * (size_t)n * n);
    uint32_t *p = (uint32_t *)malloc(sizeof(uint32_t) * n), *lab = (uint32_t *)malloc(sizeof(uint32_t) * n);
    uint64_t *rowpre = (uint64_t *)malloc(sizeof(uint64_t) * n);
    for (uint64_t round = 0;; round++) {
        uint64_t W = 0;
        for (uint32_t a = 0; a < dim; a++) {
            uint64_t s = 0;
            const uint64_t *row = g + (size_t)a * dim;
            for (uint32_t b = 0; b < dim; b++) s += row[b];
            W += s;
            rowpre[a] = W; /* inclusive prefix of row sums */
        }
        if (W == 0) break;
        for (uint32_t i = 0; i < dim; i++) p[i] = i;
        uint32_t count = dim;
        for (uint64_t d = 0; d < dim && count > target; d++) {
            uint64_t y = mulhi64(orc_draw64(key, round, d), W);
            /* first row whose inclusive prefix exceeds y */
            uint32_t lo = 0, hi = dim - 1;
            while (lo < hi) { uint32_t mid = (lo + hi) / 2; if (rowpre[mid] > y) hi = mid; else lo = mid + 1; }
            uint32_t a = lo;
            uint64_t rem = y - (a ? rowpre[a - 1] : 0);
            const uint64_t *row = g + (size_t)a * dim;
            uint32_t b = 0;
            uint64_t acc = 0;
            for (; b < dim; b++) { acc += row[b]; if (acc > rem) break; }
            uint32_t ra = qfind(p, a), rb = qfind(p, b);
            if (ra != rb) { if (ra < rb) p[rb] = ra; else p[ra] = rb; count--; }
        }
        uint32_t k = rank_labels(dim, p, lab);
        uint64_t *q = quotient(dim, g, lab, k);
        free(g);
        g = q;
        dim = k;
        if (dim <= target) break;
    }
    free(p); free(lab); free(rowpre);
    *n_out = dim;
    return g;
}

static uint64_t ks_node(uint32_t n, const uint64_t *g, uint32_t seed_r, uint32_t trial, uint64_t h) {
    if (n <= 128) {
        uint64_t *c = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n * n);
        memcpy(c, g, sizeof(uint64_t) * (size_t)n * n);
        uint64_t r = orc_stoer_wagner_dense(n, c);
        free(c);
        return r;
    }
    uint64_t W = 0;
    for (size_t i = 0; i < (size_t)n * n; i++) W += g[i];
    if (W == 0) return 0;
    uint32_t target = (uint32_t)orc_ks_target((int)n);
    uint64_t best = U64MAX;
    for (uint64_t c = 0; c < 2; c++) {
        uint64_t child = 2 * h + c;
        uint64_t key[4] = {seed_r, trial, 1 + child, 0};
        uint32_t k;
        uint64_t *q = ks_shrink(n, g, target, key, &k);
        uint64_t r = ks_node(k, q, seed_r, trial, child);
        free(q);
        if (r < best) best = r;
    }
    return best;
}

uint64_t orc_ks_dense(uint32_t n, const uint64_t *mat, uint32_t seed, uint32_t rank, uint32_t trial) {
    if (n < 2) return U64MAX;
    uint64_t ub = U64MAX;
    for (uint32_t a = 0; a < n; a++) {
        uint64_t s = 0;
        for (uint32_t b = 0; b < n; b++) s += mat[(size_t)a * n + b];
        if (s < ub) ub = s;
    }
    uint64_t r = ks_node(n, mat, seed + rank, trial, 1);
    return r < ub ? r : ub;
}

uint32_t orc_shrink_to_dense(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w,
                             uint32_t target, uint32_t seed, uint32_t rank, uint32_t trial, uint64_t *mat_out) {
    uint32_t *p = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    for (uint32_t i = 0; i < n; i++) p[i] = i;
    uint32_t count = n;
    if (target < n) {
        uint64_t key[4] = {(uint32_t)(seed + rank), trial, 1, 0};
        uint64_t *pre = (uint64_t *)malloc(sizeof(uint64_t) * (m ? m : 1));
        for (uint64_t round = 0; count > target; round++) {
            uint64_t W = 0;
            for (uint64_t e = 0; e < m; e++) {
                if (qfind(p, u[e]) != qfind(p, v[e])) W += w[e];
                pre[e] = W;
            }
            if (W == 0) break;
            uint32_t start = count;
            for (uint64_t d = 0; d < start && count > target; d++) {
                uint64_t y = mulhi64(orc_draw64(key, round, d), W);
                uint64_t lo = 0, hi = m - 1;
                while (lo < hi) { uint64_t mid = (lo + hi) / 2; if (pre[mid] > y) hi = mid; else lo = mid + 1; }
                uint32_t ra = qfind(p, u[lo]), rb = qfind(p, v[lo]);
                if (ra != rb) { if (ra < rb) p[rb] = ra; else p[ra] = rb; count--; }
            }
        }
        free(pre);
    }
    uint32_t *lab = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    uint32_t k = rank_labels(n, p, lab);
    if (mat_out) {
        memset(mat_out, 0, sizeof(uint64_t) * (size_t)k * k);
        for (uint64_t e = 0; e < m; e++) {
            uint32_t a = lab[u[e]], b = lab[v[e]];
            if (a == b) continue;
            mat_out[(size_t)a * k + b] += w[e];
            mat_out[(size_t)b * k + a] += w[e];
        }
    }
    free(p); free(lab);
    return k;
}

/* ------------------------------------------------------------------ sparse Karger-Stein nodes
 * libcac's definition of the sparse part of a trial (the reference's sparse recursion,
 * co_mincut.h:131-155 and 401-405, contracts a sparse node by exponential edge scores and a prefix
 * connected components; libcac contracts it by the same weighted rounds as Stage 1):
 *   - a node is kept as an edge list when it has more than the dense limit (16384 vertices, or
 *     the value set with orc_set_dense_limit) or, above 2048 vertices, fewer than N^2 / 32 edges;
 *     otherwise it becomes the dense matrix of the dense recursion above;
 *   - the child with heap index c of a sparse node contracts the node's edge list to
 *     max(ceil(N / sqrt 2) + 1, 128) vertices by the Stage 1 rounds with key (k0, trial, 1 + c, 0)
 *     (weighted draws over the edges that are not loops at the start of each round, in the
 *     list's order; contracted in draw order; early stop when no edge is left);
 *   - the child's edge list: every edge relabelled by rank-of-minimum labels, loops dropped,
 *     sorted by (smaller end, larger end), equal pairs merged with their weights summed
 *     (WeightedIteratedSparseSampling::reduce and SamplingSorter, sparse_graph::relabel/compact);
 *   - a node without edges has cut 0; a sparse root (plain Karger-Stein on a sparse graph, or a
 *     square_root trial whose contracted size is above the dense limit) also delivers its minimum
 *     weighted degree. The root of plain Karger-Stein is the input edge list as given. */
static uint32_t g_dense_limit = 16384;
void orc_set_dense_limit(uint32_t n) { g_dense_limit = n < 128 ? 128 : n; }

typedef struct { uint32_t n; uint64_t m; uint32_t *a, *b; uint64_t *w; } sgraph;
static void sg_free(sgraph *g) { free(g->a); free(g->b); free(g->w); }

static int is_dense(uint32_t n, uint64_t m) {
    return n <= g_dense_limit && (n <= 2048 || 32 * m >= (uint64_t)n * n);
}

/* Stage 1 rounds on an edge list with u64 weights and key `key`: labels (rank of the smallest
 * member) to lab, returns the vertex count left */
static uint32_t stage1_dpr(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint64_t *w,
                           uint32_t target, const uint64_t key[4], uint32_t *lab, uint32_t dpr);
static uint32_t stage1(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint64_t *w,
                       uint32_t target, const uint64_t key[4], uint32_t *lab) {
    return stage1_dpr(n, m, u, v, w, target, key, lab, 0);
}
/* dpr: draws per round (0: the round's vertex count) */
static uint32_t stage1_dpr(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint64_t *w,
                           uint32_t target, const uint64_t key[4], uint32_t *lab, uint32_t dpr) {
    uint32_t *p = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    for (uint32_t i = 0; i < n; i++) p[i] = i;
    uint32_t count = n;
    uint64_t *pre = (uint64_t *)malloc(sizeof(uint64_t) * (m ? m : 1));
    for (uint64_t round = 0; count > target; round++) {
        uint64_t W = 0;
        for (uint64_t e = 0; e < m; e++) {
            if (qfind(p, u[e]) != qfind(p, v[e])) W += w[e];
            pre[e] = W;
        }
        if (W == 0) break;
        uint32_t start = dpr ? dpr : count;
        for (uint64_t d = 0; d < start && count > target; d++) {
            uint64_t y = mulhi64(orc_draw64(key, round, d), W);
            uint64_t lo = 0, hi = m - 1;
            while (lo < hi) { uint64_t mid = (lo + hi) / 2; if (pre[mid] > y) hi = mid; else lo = mid + 1; }
            uint32_t ra = qfind(p, u[lo]), rb = qfind(p, v[lo]);
            if (ra != rb) { if (ra < rb) p[rb] = ra; else p[ra] = rb; count--; }
        }
    }
    free(pre);
    uint32_t k = rank_labels(n, p, lab);
    free(p);
    return k;
}

typedef struct { uint64_t key, w; } kw;
static int kw_cmp(const void *x, const void *y) {
    const uint64_t a = ((const kw *)x)->key, b = ((const kw *)y)->key;
    return a < b ? -1 : a > b;
}

/* relabel (lab may be NULL: identity), drop loops, sort by (smaller, larger end), merge */
static void merge_child(uint64_t m, const uint32_t *u, const uint32_t *v, const uint64_t *w, const uint32_t *lab,
                        uint32_t k, sgraph *out) {
    kw *e = (kw *)malloc(sizeof(kw) * (m ? m : 1));
    uint64_t c = 0;
    for (uint64_t i = 0; i < m; i++) {
        uint32_t x = lab ? lab[u[i]] : u[i], y = lab ? lab[v[i]] : v[i];
        if (x == y) continue;
        uint32_t lo = x < y ? x : y, hi = x ^ y ^ lo;
        e[c].key = (uint64_t)lo * k + hi;
        e[c].w = w[i];
        c++;
    }
    qsort(e, c, sizeof(kw), kw_cmp);
    out->n = k;
    out->a = (uint32_t *)malloc(sizeof(uint32_t) * (c ? c : 1));
    out->b = (uint32_t *)malloc(sizeof(uint32_t) * (c ? c : 1));
    out->w = (uint64_t *)malloc(sizeof(uint64_t) * (c ? c : 1));
    uint64_t j = 0;
    for (uint64_t i = 0; i < c; i++) {
        if (j && (uint64_t)out->a[j - 1] * k + out->b[j - 1] == e[i].key) { out->w[j - 1] += e[i].w; continue; }
        out->a[j] = (uint32_t)(e[i].key / k);
        out->b[j] = (uint32_t)(e[i].key % k);
        out->w[j] = e[i].w;
        j++;
    }
    out->m = j;
    free(e);
}

static uint64_t *dense_of(const sgraph *g) {
    uint64_t *mat = (uint64_t *)calloc((size_t)g->n * g->n, sizeof(uint64_t));
    for (uint64_t i = 0; i < g->m; i++) {
        mat[(size_t)g->a[i] * g->n + g->b[i]] += g->w[i];
        mat[(size_t)g->b[i] * g->n + g->a[i]] += g->w[i];
    }
    return mat;
}

static uint64_t min_degree(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint64_t *w) {
    uint64_t *deg = (uint64_t *)calloc(n ? n : 1, sizeof(uint64_t));
    for (uint64_t e = 0; e < m; e++) if (u[e] != v[e]) { deg[u[e]] += w[e]; deg[v[e]] += w[e]; }
    uint64_t best = U64MAX;
    for (uint32_t i = 0; i < n; i++) if (deg[i] < best) best = deg[i];
    free(deg);
    return best;
}

static uint64_t ks_sparse(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint64_t *w,
                          uint32_t seed_r, uint32_t trial, uint64_t h) {
    if (m == 0) return 0;
    uint32_t target = (uint32_t)orc_ks_target((int)n);
    uint32_t *lab = (uint32_t *)malloc(sizeof(uint32_t) * n);
    uint64_t best = U64MAX;
    for (uint64_t c = 0; c < 2; c++) {
        uint64_t child = 2 * h + c;
        uint64_t key[4] = {seed_r, trial, 1 + child, 0};
        uint32_t k = stage1(n, m, u, v, w, target, key, lab);
        sgraph ch;
        merge_child(m, u, v, w, lab, k, &ch);
        uint64_t r;
        if (ch.m == 0) {
            r = 0;
        } else if (is_dense(k, ch.m)) {
            uint64_t *mat = dense_of(&ch);
            r = ks_node(k, mat, seed_r, trial, child);
            free(mat);
        } else {
            r = ks_sparse(k, ch.m, ch.a, ch.b, ch.w, seed_r, trial, child);
        }
        sg_free(&ch);
        if (r < best) best = r;
    }
    free(lab);
    return best;
}

/* one trial of a sparse root (already in its list form) */
static uint64_t sparse_root(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint64_t *w,
                            uint32_t seed_r, uint32_t trial) {
    uint64_t ub = min_degree(n, m, u, v, w);
    uint64_t r = ks_sparse(n, m, u, v, w, seed_r, trial, 1);
    return r < ub ? r : ub;
}

static uint64_t *widen(uint64_t m, const uint32_t *w) {
    uint64_t *x = (uint64_t *)malloc(sizeof(uint64_t) * (m ? m : 1));
    for (uint64_t i = 0; i < m; i++) x[i] = w[i];
    return x;
}

uint64_t orc_mincut_trial(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w,
                          uint32_t seed, uint32_t rank, uint32_t trial) {
    if (n < 2) return U64MAX;
    uint32_t t = orc_intermediate_size(n, m);
    if (t > g_dense_limit) {
        /* Stage 1 to t, then the sparse root: the contracted graph merged by the device sort */
        uint64_t *w64 = widen(m, w);
        uint32_t *lab = (uint32_t *)malloc(sizeof(uint32_t) * n);
        uint64_t key[4] = {(uint32_t)(seed + rank), trial, 1, 0};
        uint32_t k = t < n ? stage1(n, m, u, v, w64, t, key, lab) : n;
        sgraph root;
        merge_child(m, u, v, w64, t < n ? lab : NULL, k, &root);
        uint64_t r = (k < 2 || root.m == 0) ? 0 : sparse_root(k, root.m, root.a, root.b, root.w, seed + rank, trial);
        sg_free(&root);
        free(lab); free(w64);
        return r;
    }
    uint64_t *mat = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(t < n ? n : t) * (t < n ? n : t));
    uint32_t k = orc_shrink_to_dense(n, m, u, v, w, t, seed, rank, trial, mat);
    uint64_t r = k < 2 ? 0 : orc_ks_dense(k, mat, seed, rank, trial);
    free(mat);
    return r;
}

/* ------------------------------------------------------------------ the group variant
 * SquareRootCut's high-concurrency variant (SquareRootCut.cpp:188-298), chosen when the virtual
 * ranks are at least twice the trial count: group_size = 2^floor(log2(p / T)) ranks share one
 * trial, so there are p / group_size trials. libcac's group trial g: WeightedIteratedSparseSampling
 * ::shrink (WeightedIteratedSparseSampling.cpp:4-24, edgesToSamplePerProcessor .hpp:66-84) as
 * Stage 1 rounds of a fixed floor(n^1.05) weighted draws each (not the round's vertex count),
 * contracted in draw order until t vertices remain, key (seed + g, 0, 1, 0); its contracted graph
 * (dense, or a sparse root above the dense limit); then, as parallel_cut(.., 2, ..) runs two
 * recursive contractions of the group's graph (recursive_contract.cpp:45-83), two Karger-Stein
 * recursions from that root, with keys (seed + g, 0, 1 + h, 0) and (seed + g, 1, 1 + h, 0). The
 * trial's value is the minimum of both and the root's minimum weighted degree. */
uint32_t orc_group_count(uint32_t ranks, uint32_t trials) {
    uint32_t per = trials ? ranks / trials : ranks;
    uint32_t size = 1;
    while (size * 2 <= per) size *= 2;
    return ranks / size;
}

uint32_t orc_group_draws(uint32_t n) { return (uint32_t)powf((float)n, 1.0f + 0.1f / 2.0f); }

uint64_t orc_mincut_group_trial(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w,
                                uint32_t seed, uint32_t group) {
    if (n < 2) return U64MAX;
    uint32_t t = orc_intermediate_size(n, m);
    uint64_t *w64 = widen(m, w);
    uint32_t *lab = (uint32_t *)malloc(sizeof(uint32_t) * n);
    uint64_t key[4] = {(uint32_t)(seed + group), 0, 1, 0};
    uint32_t k = t < n ? stage1_dpr(n, m, u, v, w64, t, key, lab, orc_group_draws(n)) : n;
    sgraph root;
    merge_child(m, u, v, w64, t < n ? lab : NULL, k, &root);
    uint64_t r = U64MAX;
    if (k < 2 || root.m == 0) {
        r = 0;
    } else if (t <= g_dense_limit) {
        uint64_t *mat = dense_of(&root);
        for (uint32_t j = 0; j < 2; j++) {
            uint64_t c = orc_ks_dense(k, mat, seed, group, j);
            if (c < r) r = c;
        }
        free(mat);
    } else {
        for (uint32_t j = 0; j < 2; j++) {
            uint64_t c = sparse_root(k, root.m, root.a, root.b, root.w, seed + group, j);
            if (c < r) r = c;
        }
    }
    sg_free(&root);
    free(lab); free(w64);
    return r;
}

/* one trial of plain Karger-Stein on the whole graph (the karger_stein executable): the root is
 * dense (the n x n matrix) or sparse (the input edge list as given) by the rule above */
uint64_t orc_ks_trial(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w, uint32_t seed,
                      uint32_t trial) {
    if (n < 2) return U64MAX;
    if (is_dense(n, m)) {
        uint64_t *mat = (uint64_t *)calloc((size_t)n * n, sizeof(uint64_t));
        for (uint64_t e = 0; e < m; e++) {
            if (u[e] == v[e]) continue;
            mat[(size_t)u[e] * n + v[e]] += w[e];
            mat[(size_t)v[e] * n + u[e]] += w[e];
        }
        uint64_t r = orc_ks_dense(n, mat, seed, 0, trial);
        free(mat);
        return r;
    }
    uint64_t *w64 = widen(m, w);
    uint64_t r = sparse_root(n, m, u, v, w64, seed, trial);
    free(w64);
    return r;
}

uint64_t orc_square_root(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w,
                         double p, uint32_t seed, uint32_t ranks, uint32_t *per_rank_out) {
    if (ranks == 0) ranks = 1;
    double total = orc_number_of_trials(n, m, p);
    const int high = (double)ranks >= 2.0 * total; /* SquareRootCut::lowConcurrency (SquareRootCut.cpp:11-13) */
    uint32_t per = high ? 1 : (uint32_t)ceil(total / ranks);
    if (per_rank_out) *per_rank_out = per;
    /* the answer also takes the graph's minimum weighted degree (a single-vertex cut): libcac's
       square_root reports min(that, every trial), so a query whose trials all contracted the
       minimum-degree vertex still reports a minimum cut that is a single-vertex cut */
    uint64_t *deg = (uint64_t *)calloc(n ? n : 1, sizeof(uint64_t));
    for (uint64_t e = 0; e < m; e++) if (u[e] != v[e]) { deg[u[e]] += w[e]; deg[v[e]] += w[e]; }
    uint64_t best = U64MAX;
    for (uint32_t i = 0; i < n; i++) if (deg[i] < best) best = deg[i];
    free(deg);
    if (high) {
        uint32_t groups = orc_group_count(ranks, (uint32_t)total);
        for (uint32_t g = 0; g < groups; g++) {
            uint64_t c = orc_mincut_group_trial(n, m, u, v, w, seed, g);
            if (c < best) best = c;
        }
        return best;
    }
    for (uint32_t r = 0; r < ranks; r++)
        for (uint32_t i = 0; i < per; i++) {
            uint64_t c = orc_mincut_trial(n, m, u, v, w, seed, r, i);
            if (c < best) best = c;
        }
    return best;
}
