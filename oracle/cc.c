/*
 * ORACLE (test infrastructure) — connected components.
 *
 * orc_cc_labels: the closed form of the reference's CC output. The reference relabels the
 * vertices of every round by first appearance over j = 0..n-1
 * (src/IteratedSparseSampling.hpp:210-220) and composes the maps across rounds
 * (src/UnweightedIteratedSparseSampling.cpp:60-62); both steps preserve the order of
 * component minima, so the final label of v is the rank of min(component(v)) among all
 * component minima. Computed here with a plain union-find over every edge.
 *
 * orc_cc_iss: a step-by-step restatement of the reference's iterated-sparse-sampling loop,
 * kept as the CPU baseline of the same work (sampling, gather, shuffle, prefix union-find,
 * relabel, slice rewrite). Its labels must equal orc_cc_labels for every seed.
 */
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "oracle.h"

static uint32_t uf_find_halving(uint32_t *p, uint32_t x) {
    while (p[x] != x) {
        p[x] = p[p[x]];
        x = p[x];
    }
    return x;
}

uint32_t orc_cc_labels(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, uint32_t *labels) {
    uint32_t *p = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    for (uint32_t i = 0; i < n; i++) p[i] = i;
    for (uint64_t e = 0; e < m; e++) {
        uint32_t a = uf_find_halving(p, u[e]), b = uf_find_halving(p, v[e]);
        if (a == b) continue;
        if (a < b) p[b] = a; else p[a] = b; /* the smaller id stays root */
    }
    uint32_t count = 0;
    for (uint32_t i = 0; i < n; i++) {
        uint32_t r = uf_find_halving(p, i);
        if (r == i) { if (labels) labels[i] = count; count++; }
        else if (labels) labels[i] = labels[r]; /* r < i, already labelled */
    }
    free(p);
    return count;
}

/* ---- restatement of the reference's ISS CC ---- */

typedef struct { uint32_t from, to; } edge2;

/* sitmo::prng_engine(seed) as a sequential 32-bit stream (lib/prng_engine.hpp:195-212). */
typedef struct { uint64_t key[4]; uint64_t block; uint64_t out[4]; unsigned pos; } seq_engine;

static void eng_init(seq_engine *e, uint32_t seed) {
    memset(e, 0, sizeof(*e));
    e->key[0] = seed;
    e->pos = 8; /* forces a block computation at the first call */
    e->block = (uint64_t)-1;
}

static uint32_t eng_next(seq_engine *e) {
    if (e->pos == 8) {
        e->block++;
        uint64_t ctr[4] = {e->block, 0, 0, 0};
        orc_sitmo_block(e->key, ctr, e->out);
        e->pos = 0;
    }
    unsigned k = e->pos++;
    uint64_t w = e->out[k >> 1];
    return (k & 1) ? (uint32_t)(w >> 32) : (uint32_t)w;
}

/* union by rank + full path compression (the algorithm of the Boost disjoint_sets the
 * reference wraps in src/DisjointSets.hpp:7-42) */
static uint32_t ds_find(uint32_t *parent, uint32_t x) {
    uint32_t r = x;
    while (parent[r] != r) r = parent[r];
    while (parent[x] != r) { uint32_t nx = parent[x]; parent[x] = r; x = nx; }
    return r;
}
static void ds_link(uint32_t *parent, uint8_t *rank, uint32_t a, uint32_t b) {
    if (rank[a] > rank[b]) parent[b] = a;
    else { parent[a] = b; if (rank[a] == rank[b]) rank[b]++; }
}

uint64_t orc_cc_sample_count(uint32_t n, uint64_t edges_left) {
    /* unsigned(std::pow((float)n0, 1 + eps/2) * (1 + delta)), eps = 0.09f, delta = 0.2f */
    uint64_t s = (uint64_t)(uint32_t)(powf((float)n, 1.0f + 0.09f / 2) * (1.0f + 0.2f));
    return s < edges_left ? s : edges_left;
}

/* UnweightedIteratedSparseSampling::edgesToSamplePerProcessor (.cpp:80-128), uint32 wraps kept */
static void edges_to_sample(uint32_t n0, uint32_t ranks, const int *avail, int *per) {
    uint32_t total = 0;
    for (uint32_t i = 0; i < ranks; i++) total += (uint32_t)avail[i];
    uint32_t want = (uint32_t)(powf((float)n0, 1.0f + 0.09f / 2) * (1.0f + 0.2f));
    uint32_t to_sample = want < total ? want : total;
    uint32_t threshold = (uint32_t)(3.0f / (0.2f * 0.2f) * logf((float)ranks / 0.9f));
    uint32_t remaining = to_sample;
    for (uint32_t i = 0; i < ranks; i++) per[i] = 0;
    for (uint32_t i = 0; i < ranks; i++) {
        if ((uint32_t)avail[i] <= threshold) {
            per[i] = avail[i];
            remaining -= (uint32_t)avail[i];
            to_sample -= (uint32_t)avail[i];
        }
    }
    for (uint32_t i = 0; i < ranks; i++) {
        if (per[i] != 0) continue;
        int share = (int)((float)to_sample * (float)avail[i] / (float)total);
        per[i] = share < avail[i] ? share : avail[i];
        remaining -= (uint32_t)per[i];
    }
    for (uint32_t sp = 0; remaining > 0 && sp < ranks; sp++) {
        if (avail[sp] > per[sp]) {
            uint32_t room = (uint32_t)(avail[sp] - per[sp]);
            uint32_t delta = room < remaining ? room : remaining;
            per[sp] += (int)delta;
            remaining -= delta;
        }
    }
}

/* The per-rank phases of a round (slice load, sampling, slice rewrite) run on `threads` host
 * threads, rank r on thread r mod threads, as the reference's MPI ranks run them side by side;
 * the root's gather, shuffle, prefix union-find and relabelling stay sequential. */
typedef struct {
    uint32_t ranks, threads, t, phase, n;
    const uint32_t *u, *v, *map;
    edge2 **sl;
    uint64_t *len, *off;
    uint64_t portion, m;
    seq_engine *eng;
    const int *per;
    edge2 *gs;
} rank_job;

static void rank_phase(rank_job *J, uint32_t r) {
    if (J->phase == 0) { /* load the slice as {from, to} records */
        uint64_t from = J->portion * r;
        for (uint64_t e = 0; e < J->len[r]; e++) { J->sl[r][e].from = J->u[from + e]; J->sl[r][e].to = J->v[from + e]; }
    } else if (J->phase == 1) { /* sample (.cpp:24-37) into the rank's place of the gather */
        edge2 *dst = J->gs + J->off[r];
        if ((uint64_t)J->per[r] == J->len[r]) {
            memcpy(dst, J->sl[r], sizeof(edge2) * J->len[r]);
        } else {
            for (int k = 0; k < J->per[r]; k++) {
                uint64_t idx = eng_next(&J->eng[r]) % (uint32_t)J->len[r];
                dst[k] = J->sl[r][idx];
            }
        }
    } else { /* rewrite the slice and drop loops (IteratedSparseSampling.hpp:160-172) */
        uint64_t w = 0;
        for (uint64_t e = 0; e < J->len[r]; e++) {
            uint32_t a = J->map[J->sl[r][e].from], b = J->map[J->sl[r][e].to];
            if (a != b) { J->sl[r][w].from = a; J->sl[r][w].to = b; w++; }
        }
        J->len[r] = w;
    }
}

static void *rank_worker(void *arg) {
    rank_job *J = (rank_job *)arg;
    for (uint32_t r = J->t; r < J->ranks; r += J->threads) rank_phase(J, r);
    return NULL;
}

static void run_ranks(rank_job *base, uint32_t phase) {
    uint32_t T = base->threads < base->ranks ? base->threads : base->ranks;
    if (T <= 1) {
        base->phase = phase;
        for (uint32_t r = 0; r < base->ranks; r++) rank_phase(base, r);
        return;
    }
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * T);
    rank_job *jobs = (rank_job *)malloc(sizeof(rank_job) * T);
    uint32_t started = 0;
    for (uint32_t t = 0; t < T; t++) {
        jobs[t] = *base;
        jobs[t].phase = phase;
        jobs[t].t = t;
        jobs[t].threads = T;
        if (pthread_create(&th[t], NULL, rank_worker, &jobs[t]) == 0) started++;
        else { jobs[t].threads = T; rank_worker(&jobs[t]); th[t] = 0; } /* run it here */
    }
    for (uint32_t t = 0; t < T; t++) if (th[t]) pthread_join(th[t], NULL);
    (void)started;
    free(th); free(jobs);
}

uint32_t orc_cc_iss(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, uint32_t seed, uint32_t ranks,
                    uint32_t *labels, uint32_t *rounds_out) {
    return orc_cc_iss_mt(n, m, u, v, seed, ranks, 1, labels, rounds_out);
}

uint32_t orc_cc_iss_mt(uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, uint32_t seed, uint32_t ranks,
                       uint32_t threads, uint32_t *labels, uint32_t *rounds_out) {
    if (ranks == 0) ranks = 1;
    if (threads == 0) threads = 1;
    /* slices: rank r owns lines [r*floor(m/P), (r+1)*floor(m/P)), the last rank the rest
     * (UnweightedIteratedSparseSampling.cpp:5-21) */
    /* slices hold {from, to} records like the reference's UnweightedGraph::Edge (8 bytes) */
    edge2 **sl = (edge2 **)calloc(ranks, sizeof(edge2 *));
    uint64_t *len = (uint64_t *)calloc(ranks, sizeof(uint64_t));
    seq_engine *eng = (seq_engine *)calloc(ranks, sizeof(seq_engine));
    uint64_t portion = m / ranks;
    for (uint32_t r = 0; r < ranks; r++) {
        uint64_t from = portion * r, to = (r == ranks - 1) ? m : portion * (r + 1);
        len[r] = to - from;
        sl[r] = (edge2 *)malloc(sizeof(edge2) * (len[r] ? len[r] : 1));
        eng_init(&eng[r], seed + r);
    }
    uint64_t *off = (uint64_t *)calloc(ranks, sizeof(uint64_t));
    rank_job job;
    memset(&job, 0, sizeof(job));
    job.ranks = ranks; job.threads = threads; job.n = n; job.u = u; job.v = v; job.sl = sl; job.len = len;
    job.off = off; job.portion = portion; job.m = m; job.eng = eng;
    run_ranks(&job, 0);
    uint32_t *comp = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    for (uint32_t i = 0; i < n; i++) comp[i] = i;
    uint32_t vcount = n, rounds = 0;
    int *avail = (int *)malloc(sizeof(int) * ranks), *per = (int *)malloc(sizeof(int) * ranks);
    uint32_t *parent = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    uint8_t *rk = (uint8_t *)malloc(n ? n : 1);
    int64_t *lab = (int64_t *)malloc(sizeof(int64_t) * (n ? n : 1));
    uint32_t *map = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));

    for (;;) {
        uint64_t left = 0;
        for (uint32_t r = 0; r < ranks; r++) left += len[r];
        if (left == 0) break;
        rounds++;
        for (uint32_t r = 0; r < ranks; r++) avail[r] = (int)len[r];
        edges_to_sample(n, ranks, avail, per);
        uint64_t total = 0;
        for (uint32_t r = 0; r < ranks; r++) total += (uint64_t)per[r];
        /* sample (.cpp:24-37) and gather in rank order (IteratedSparseSampling.hpp:261-271) */
        edge2 *gs = (edge2 *)malloc(sizeof(edge2) * (total ? total : 1));
        uint64_t at = 0;
        for (uint32_t r = 0; r < ranks; r++) { off[r] = at; at += (uint64_t)per[r]; }
        job.per = per; job.gs = gs;
        run_ranks(&job, 1);
        /* shuffle with the root's engine (IteratedSparseSampling.hpp:278). Fisher-Yates with
         * multiply-shift draws: libstdc++'s std::shuffle consumes the engine differently, which
         * only changes the order in which the prefix union-find meets the samples, never the
         * labels (the target is a single component). */
        for (uint64_t i = total; i > 1; i--) {
            uint64_t j = ((uint64_t)eng_next(&eng[0]) * i) >> 32;
            edge2 t = gs[i - 1]; gs[i - 1] = gs[j]; gs[j] = t;
        }
        /* prefix union-find to one component (IteratedSparseSampling.hpp:182-224) */
        for (uint32_t i = 0; i < vcount; i++) { parent[i] = i; rk[i] = 0; }
        uint32_t active = vcount;
        for (uint64_t i = 0; i < total && active > 1; i++) {
            uint32_t a = ds_find(parent, gs[i].from), b = ds_find(parent, gs[i].to);
            if (a != b) { active--; ds_link(parent, rk, a, b); }
        }
        for (uint32_t j = 0; j < vcount; j++) lab[j] = -1;
        uint32_t next = 0;
        for (uint32_t j = 0; j < vcount; j++) {
            uint32_t r = ds_find(parent, j);
            if (lab[r] < 0) lab[r] = next++;
            map[j] = (uint32_t)lab[r];
        }
        for (uint32_t i = 0; i < n; i++) comp[i] = map[comp[i]];
        /* every rank rewrites its slice and drops loops (IteratedSparseSampling.hpp:160-172) */
        job.map = map;
        run_ranks(&job, 2);
        vcount = active;
        free(gs);
    }
    if (labels) memcpy(labels, comp, sizeof(uint32_t) * n);
    if (rounds_out) *rounds_out = rounds;
    for (uint32_t r = 0; r < ranks; r++) free(sl[r]);
    free(sl); free(len); free(eng); free(comp); free(avail); free(per); free(off);
    free(parent); free(rk); free(lab); free(map);
    return vcount;
}
