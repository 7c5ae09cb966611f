// Internal declarations shared by the libcac translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <set>
#include <vector>

#include "../../include/cac.h"

namespace cac {

// Thread-local last-error message (cac_last_error).
void set_error(const std::string &msg);

#define CAC_CUDA_TRY(expr)                                                                        \
    do {                                                                                          \
        cudaError_t _e = (expr);                                                                  \
        if (_e != cudaSuccess) {                                                                  \
            ::cac::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));                 \
            return CAC_ERR_CUDA;                                                                  \
        }                                                                                         \
    } while (0)

#define CAC_TRY(expr)                                                                             \
    do {                                                                                          \
        int _s = (expr);                                                                          \
        if (_s != CAC_OK) return _s;                                                              \
    } while (0)

// A grow-only device scratch arena owned by a ctx (reset per call, never shrunk).
struct Arena {
    char *base = nullptr;
    size_t cap = 0;
    size_t used = 0;
};

}  // namespace cac

struct cac_graph;

namespace cac {
// Identity of a connected-components query whose launch sequence is cached as a CUDA graph.
struct CCGraphKey {
    const void *u = nullptr, *v = nullptr, *labels = nullptr;
    uint32_t n = 0;
    uint64_t m = 0;
    uint32_t seed = 0, ranks = 0;
    const void *arena_base = nullptr;
    size_t arena_cap = 0;
};
}  // namespace cac

struct cac_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    uint64_t budget = 0;     // 0: unlimited
    uint64_t held = 0;       // device bytes held (graphs + arena)
    int num_sms = 0;
    cac::Arena arena;  // kernel scratch
    cac::Arena io;     // staging for host-buffer entry points
    cudaEvent_t ev[8] = {};  // phase timing events
    std::set<cac_graph *> graphs;    // live graphs, released by cac_ctx_destroy
    cac::CCGraphKey cc_key;          // last connected-components query
    cudaGraphExec_t cc_exec = nullptr;  // its captured launch sequence (second sighting onwards)
    uint32_t *pinned_u32 = nullptr;  // 64 KB pinned staging: [0,256) B scalar results, then descriptors
};

struct cac_graph {
    cac_ctx *ctx = nullptr;
    uint32_t n = 0;
    uint64_t m = 0;
    uint64_t total_weight = 0;
    uint32_t *u = nullptr;  // device, m entries
    uint32_t *v = nullptr;  // device, m entries
    uint32_t *w = nullptr;  // device, m entries (all ones when the input had no weights)
    uint64_t bytes = 0;
};

namespace cac {

// Device memory accounting against the ctx budget.
int dev_alloc(cac_ctx *ctx, void **p, size_t bytes);
void dev_free(cac_ctx *ctx, void *p, size_t bytes);
// Scratch arena: reset, then carve aligned chunks (grows by reallocating when too small;
// growing invalidates earlier chunks, so callers size everything before carving).
int arena_reserve(cac_ctx *ctx, Arena &a, size_t bytes);
void *arena_take(Arena &a, size_t bytes);
inline int arena_reserve(cac_ctx *ctx, size_t bytes) { return arena_reserve(ctx, ctx->arena, bytes); }
inline void *arena_take(cac_ctx *ctx, size_t bytes) { return arena_take(ctx->arena, bytes); }
inline void arena_reset(cac_ctx *ctx) { ctx->arena.used = 0; }
inline size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

// ---- CC (cc.cu) ----
struct CCPlan {
    // per virtual rank: slice offset/length in the edge array and number of draws
    std::vector<uint64_t> slice_off, slice_len, draws;
};
CCPlan cc_plan(uint32_t n, uint64_t m, uint32_t ranks);
int cc_run(cac_ctx *ctx, uint32_t n, uint64_t m, const uint32_t *d_u, const uint32_t *d_v, uint32_t seed,
           uint32_t ranks, uint32_t *d_labels, cac_cc_result *res);
size_t cc_scratch_bytes(uint32_t n, uint32_t ranks, uint64_t m);
void cc_graph_reset(cac_ctx *ctx);

// ---- min cut (mincut.cu) ----
int mincut_trials(cac_ctx *ctx, const cac_graph *g, uint32_t seed, uint32_t ranks, uint32_t per_rank,
                  uint64_t *d_cuts, float *device_ms);
int ks_dense_one(cac_ctx *ctx, uint32_t n, const uint64_t *mat_host, uint32_t seed, uint32_t rank, uint32_t trial,
                 uint64_t *cut);
int exact_small(cac_ctx *ctx, uint32_t n, const uint64_t *mat_host, uint64_t *cut);

// ---- approx cut (approx.cu) ----
int approx_run(cac_ctx *ctx, const cac_graph *g, double p, uint32_t seed, uint32_t ranks, cac_approx_result *res);

// ---- sitmo (sitmo_kernels.cu) ----
int sitmo_blocks(cac_ctx *ctx, const uint64_t key[4], const uint64_t ctr0[4], uint64_t nblocks, uint64_t *out_host);

// ---- trial budget (host math shared with the CLI; restated from the reference) ----
uint32_t intermediate_size(uint32_t n, uint64_t m);
uint32_t number_of_trials(uint32_t n, uint64_t m, double p);
int ks_target(int n);
double min_success_in_one_trial(int n);
uint32_t approx_copies(double p);

}  // namespace cac
