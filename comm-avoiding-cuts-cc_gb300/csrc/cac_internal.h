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
inline const char *src_base(const char *path) {
    const char *b = path;
    for (const char *c = path; *c; c++)
        if (*c == '/') b = c + 1;
    return b;
}

#define CAC_CUDA_TRY(expr)                                                                        \
    do {                                                                                          \
        cudaError_t _e = (expr);                                                                  \
        if (_e != cudaSuccess) {                                                                  \
            ::cac::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e) + " (" +          \
                             ::cac::src_base(__FILE__) + ":" + std::to_string(__LINE__) + ")");   \
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
struct CCStreamKey {
    const void *h_u = nullptr, *h_v = nullptr, *h_labels = nullptr, *d_u = nullptr, *d_v = nullptr,
               *d_labels = nullptr;
    uint32_t n = 0;
    uint64_t m = 0;
    bool zero_copy = false;
    const void *arena_base = nullptr;
    size_t arena_cap = 0;
};

struct CCGraphKey {
    const void *u = nullptr, *v = nullptr, *labels = nullptr;
    uint32_t n = 0;
    uint64_t m = 0;
    uint32_t seed = 0, ranks = 0;
    const void *arena_base = nullptr;
    size_t arena_cap = 0;
    bool check = false;
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
    cudaMemPool_t pool = nullptr;    // stream-ordered pool of the Karger-Stein level buffers (keeps its memory)
    cac::CCGraphKey cc_key;          // last connected-components query
    cac::CCStreamKey cc_stream_key;  // last host-edge (streamed) connected-components query
    cudaGraphExec_t cc_stream_exec = nullptr;  // its captured launch sequence
    cudaGraphExec_t cc_exec = nullptr;  // its captured launch sequence (second sighting onwards)
    uint32_t *pinned_u32 = nullptr;  // 64 KB pinned staging: [0,256) B scalar results, then descriptors
    void *ks_scratch = nullptr;      // grow-only Karger-Stein scratch buffers (mincut.cu)
    uint8_t quotient_choice[32] = {};  // autotuned quotient kernel per (N bucket, width); 0: untuned
    uint8_t quotient_forced = 0;       // a quotient kernel chosen by the caller instead (0: autotuned)
    bool plan_ahead = true;            // Karger-Stein levels planned at their target sizes (mincut.cu)
    uint64_t plan_redos = 0;           // runs redone level by level after a child stopped off its target
    cudaStream_t copy_stream = nullptr;  // host-to-device chunks of cac_cc_edges (created on first use)
    cudaEvent_t chunk_ev[40] = {};       // start + one per piece and gap copy in flight
    uint32_t dense_limit = 16384;        // Karger-Stein nodes above this many vertices stay edge lists
};

struct cac_graph {
    cac_ctx *ctx = nullptr;
    uint32_t n = 0;
    uint64_t m = 0;
    uint64_t total_weight = 0;
    bool unit_weights = true;  // every edge weight is 1
    uint32_t *u = nullptr;  // device, m entries
    uint32_t *v = nullptr;  // device, m entries
    uint32_t *w = nullptr;  // device, m entries (all ones when the input had no weights)
    uint64_t bytes = 0;
    // smallest weighted vertex degree (a single-vertex cut), computed on first use
    bool min_degree_known = false;
    uint64_t min_degree = 0;
};

namespace cac {

// Raise a kernel's dynamic shared-memory limit to the device's opt-in maximum, once per device.
// The limit belongs to the function, process-wide: setting it per launch to that launch's size
// would break a concurrent launch of the same kernel with a larger size from another thread, so
// it is only ever raised.
int smem_optin(cac_ctx *ctx, const void *func);
template <typename F>
inline int smem_optin(cac_ctx *ctx, F *func) {
    return smem_optin(ctx, reinterpret_cast<const void *>(func));
}

// The graph's minimum weighted degree: the cut around one vertex, an upper bound of the minimum
// cut that every square_root answer also takes (computed on ctx's stream once, then cached).
int graph_min_degree(cac_ctx *ctx, cac_graph *g, uint64_t *out);

// Device memory accounting against the ctx budget.
int dev_alloc(cac_ctx *ctx, void **p, size_t bytes);
void dev_free(cac_ctx *ctx, void *p, size_t bytes);
// Per-query temporaries, stream-ordered on the ctx stream from the ctx's pool (no device-wide
// synchronisation as with cudaFree; the pool keeps freed memory for the next query).
int stream_alloc(cac_ctx *ctx, void **p, size_t bytes);
void stream_free(cac_ctx *ctx, void *p, size_t bytes);
// Scratch arena: reset, then carve aligned chunks (grows by reallocating when too small;
// growing invalidates earlier chunks, so callers size everything before carving).
int arena_reserve(cac_ctx *ctx, Arena &a, size_t bytes);
void *arena_take(Arena &a, size_t bytes);
inline int arena_reserve(cac_ctx *ctx, size_t bytes) { return arena_reserve(ctx, ctx->arena, bytes); }
inline void *arena_take(cac_ctx *ctx, size_t bytes) { return arena_take(ctx->arena, bytes); }
inline void arena_reset(cac_ctx *ctx) { ctx->arena.used = 0; }
inline size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

// Graph from edge arrays (host or device): copies, validates ids, totals the weights.
int graph_create(cac_ctx *ctx, uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w,
                 int where, cac_graph **out);

// ---- CC (cc.cu) ----
struct CCPlan {
    // per virtual rank: slice offset/length in the edge array and number of draws
    std::vector<uint64_t> slice_off, slice_len, draws;
};
CCPlan cc_plan(uint32_t n, uint64_t m, uint32_t ranks);
// check_ids: the endpoints were not validated (caller arrays); every kernel checks them and an
// endpoint >= n fails the query with CAC_ERR_INVALID.
int cc_run(cac_ctx *ctx, uint32_t n, uint64_t m, const uint32_t *d_u, const uint32_t *d_v, uint32_t seed,
           uint32_t ranks, uint32_t *d_labels, cac_cc_result *res, bool check_ids = false);
size_t cc_scratch_bytes(uint32_t n, uint32_t ranks, uint64_t m);
// CC of an edge list in host memory: parts copied to d_u/d_v on a second stream while the ctx
// stream hooks or filters each part that has arrived (cac_cc_edges); labels copied to h_labels.
int cc_run_streamed(cac_ctx *ctx, uint32_t n, uint64_t m, const uint32_t *h_u, const uint32_t *h_v, uint32_t *d_u,
                    uint32_t *d_v, uint32_t *d_labels, uint32_t *h_labels, cac_cc_result *res);
void cc_graph_reset(cac_ctx *ctx);

// ---- min cut (mincut.cu) ----
// Stream-ordered, reference-counted device buffer holding the matrices made by one admission or
// one Karger-Stein step; freed when the last node or task reading it has been consumed.
struct MatBuf {
    void *p;
    size_t bytes;
    int refs;
};

// A Karger-Stein recursion node of one trial: its matrix and where its trial's cut goes.
struct KNode {
    uint64_t *cut;     // the trial's cut (device)
    uint32_t k0, idx;  // stream key words 0, 1 (seed + virtual rank, trial index within the rank)
    uint64_t h;        // heap index (root 1, children 2h, 2h + 1)
    uint32_t N;
    uint32_t is_root;  // roots also deliver the minimum weighted degree bound
    uint32_t small;    // entries fit in 32 bits (total graph weight < 2^32)
    uint32_t query;    // owner query (engine bookkeeping)
    const void *mat;   // N x N row-major: u32 entries when `small`, else u64
    MatBuf *buf;
    uint64_t *pre = nullptr;  // row sums (N) + 32-column block prefixes (N x ceil(N/32)), when made with the matrix
};

// A child being contracted from `src` (round > 0: continuing on the quotient of earlier rounds).
struct KTask {
    KNode src;
    uint64_t h;
    uint32_t round;
    uint32_t target;
    uint32_t src_index;
};

// Level-synchronous Karger-Stein over any set of trials of any graphs: every step solves the
// leaves, and contracts and builds the children of every other node, in a few launches. Nodes
// can be added between steps (continuous batching of queries).
class KsEngine {
  public:
    explicit KsEngine(cac_ctx *ctx);
    ~KsEngine();
    KsEngine(const KsEngine &) = delete;
    KsEngine &operator=(const KsEngine &) = delete;
    int alloc(size_t bytes, MatBuf **out);  // refs start at 0
    void release(MatBuf *b);                // drops one reference
    void add(const KNode &nd);              // takes one reference on nd.buf
    bool idle() const { return nodes_.empty() && carried_.empty(); }
    // Planning ahead: every child is taken to stop at its target size, so a step needs no read-back
    // of the children's sizes; a child that stops elsewhere (a round that ran out of draws, or a
    // source without edges) sets bit 4 of the error word and the caller redoes the run without it.
    void set_plan_ahead(bool on) { plan_ahead_ = on; }
    bool plan_ahead() const { return plan_ahead_; }
    uint32_t *err_word() const;             // the engine's device error word
    int step();
    int init_err();
    int read_err(uint32_t *err);
    std::vector<int64_t> outstanding;  // live nodes and tasks per query

  private:
    cac_ctx *ctx_;
    std::vector<KNode> nodes_;
    std::vector<KTask> carried_;
    bool release_err_ = false;
    bool plan_ahead_ = false;
    void *d_kout_, *d_prep_, *d_tscratch_, *d_err_;  // the ctx's grow-only scratch (mincut.cu)
};

// A Karger-Stein node kept as an edge list (sparse_ks.cu): a root above the dense limit, or a
// child of such a node that is still above it or has fewer than N^2 / 32 edges.
struct SparseNode {
    uint64_t *cut;            // the trial's cut (device)
    uint32_t k0, idx;         // stream key words 0, 1
    uint64_t h;               // heap index
    uint32_t N;
    uint64_t m;
    const uint32_t *a, *b;    // edge ends (device)
    const void *w;            // weights: u64 when w64, else u32
    bool w64;
    bool is_root;             // roots also deliver their minimum weighted degree
    uint32_t small;           // the query's total weight is below 2^32 (u32 matrix entries)
    uint32_t query;
    MatBuf *buf;              // owner of a, b, w (null: the input graph)
};
// Dense or sparse: the rule shared with the oracle (above the limit, or above kSmallDense vertices
// with fewer than N^2 / 32 edges: an edge list). Small nodes are dense whatever their density: the
// dense engine steps thousands of them in one launch per kernel, where edge lists would cost a
// contraction, a sort and a merge per level.
constexpr uint32_t kSmallDense = 2048;
inline bool ks_is_dense(const cac_ctx *ctx, uint32_t N, uint64_t m) {
    return N <= ctx->dense_limit && (N <= kSmallDense || 32 * m >= (uint64_t)N * N);
}
// Runs every sparse level of the given nodes (each holding one reference on its buffer): children
// contracted by the Stage 1 rounds, relabelled, sorted and merged on the device; children that
// are dense join `eng` as matrices, the others are contracted in turn.
int sparse_phase(cac_ctx *ctx, KsEngine &eng, std::vector<SparseNode> nodes);

// The status and message of a nonzero engine error word (bit 1: a bounded bulk-copy wait ran
// out; otherwise an inconsistent selection prefix).
int engine_error(uint32_t err);

struct MincutQuery {
    const cac_graph *g;
    uint32_t seed, ranks, per_rank;
    uint64_t *d_cuts;  // ranks * per_rank trial cuts (device), or `groups` of them
    uint32_t t = 0;    // contraction size before Karger-Stein (0: square_root's intermediate size)
    uint32_t groups = 0;  // > 0: the high-concurrency group variant with this many group trials
};
// The trial layout of a square_root query (SquareRootCut.cpp:11-13, 99-100, 188-215): the low-
// concurrency variant's ceil(T / ranks) trials per rank, or, when ranks >= 2 T, the group
// variant's ranks / 2^floor(log2(ranks / T)) group trials (per_rank is then 1, as the reference's
// CSV prints). Fails when the trial count passes 2^32 - 1.
struct TrialLayout {
    uint32_t per_rank, total, groups;  // groups > 0 only for the group variant
    bool high;
};
int trial_layout(const char *who, uint32_t n, uint64_t m, double p, uint32_t ranks, TrialLayout *out);
// Stage 1 and Stage 2 of several queries into a running engine (engine ids ids[i]); their
// Stage 1 trials share launches. Every trial cut starts at 2^64 - 1 and the root nodes carry the
// query's engine id; a query is done when outstanding[id] is 0.
// status[i] is each query's own result (a query that fails its checks fails alone; a failure of
// the shared admission is every admitted query's).
int mincut_admit_queries(cac_ctx *ctx, KsEngine &eng, const std::vector<MincutQuery> &qs,
                         const std::vector<uint32_t> &ids, std::vector<int> &status, std::vector<std::string> &msgs);
// Stage 1 of B trials (keys k0[b], idx[b]) of a graph with more than 16384 vertices in global
// memory (shrink_big.cu): labels to d_lab[b * n ..], vertices left to d_kout[b].
uint64_t shrink_big_scratch(uint32_t n, uint64_t m, uint32_t B);
// One contraction task of shrink_tasks: a graph (u32 or u64 weights), its target, the stream key
// (k0, idx, tag, 0) of its draws, where its labels and its vertex count go.
struct ShrinkTask {
    const uint32_t *U, *V;
    const void *W;
    bool w64;
    uint64_t m;
    uint32_t n, target;
    uint32_t k0, idx;
    uint64_t tag;
    uint32_t *lab;    // n (device)
    uint32_t *k_out;  // 1 (device)
    uint32_t dpr;     // draws per round: 0 for the round's vertex count (SequentialSquareRootCut's rounds),
                      // or a fixed count (the group variant's floor(n0^1.05) samples per round)
};
uint64_t shrink_task_scratch(uint32_t n, uint64_t m, uint32_t dpr = 0);
uint64_t shrink_tasks_scratch(const std::vector<ShrinkTask> &tasks);
int shrink_tasks(cac_ctx *ctx, const std::vector<ShrinkTask> &tasks, void *scratch);
// Device sort and merge of a relabelled edge list (sort.cu): the pairs of the non-loop edges
// (lab[a], lab[b]) over k vertices, sorted by (smaller, larger end), equal pairs merged with u64
// weight sums; *d_count (device) gets the number of pairs.
uint64_t merge_edges_scratch(uint64_t m);
template <typename WT>
int merge_edges(cac_ctx *ctx, const uint32_t *a, const uint32_t *b, const WT *w, uint64_t m, const uint32_t *lab,
                uint32_t k, uint32_t *oa, uint32_t *ob, uint64_t *ow, uint32_t *d_count, void *scratch);
int scan_u32(cac_ctx *ctx, uint32_t *x, uint64_t n, uint32_t *sums, uint32_t *total);
// One child of merge_edges_multi: its parent's edges and the labels of its contraction.
struct MergeTask {
    const uint32_t *a, *b;  // parent edge ends (device)
    const void *w;          // parent weights: u64 when w64, else u32
    uint32_t w64;
    uint32_t k;             // child vertices
    uint64_t m;             // parent edges
    const uint32_t *lab;    // parent vertex -> child label (null: identity)
    uint64_t in_off, key_off;  // filled in by merge_edges_multi
};
int merge_edges_multi(cac_ctx *ctx, std::vector<MergeTask> &tasks, uint32_t *oa, uint32_t *ob, uint64_t *ow,
                      uint32_t *counts, void *scratch);
uint64_t merge_edges_multi_scratch(uint64_t M, uint32_t B);
int shrink_big(cac_ctx *ctx, const cac_graph *g, uint32_t target, uint32_t B, const uint32_t *k0, const uint32_t *idx,
               uint32_t *d_lab, uint32_t *d_kout, void *scratch);
// Quotient kernel choices of the autotuner (cac_ctx::quotient_choice), bucketed by
// floor(log2 N) and entry width.
constexpr uint8_t kQuotientWarp = 1, kQuotientShared = 2, kQuotientBulk = 3, kQuotientRule = 4;
// Engine error word bits: 1 an inconsistent selection prefix in a contraction, 2 a bulk-copy wait
// past its bound, 4 a child planned at its target size that stopped elsewhere (the run is redone
// without planning ahead)
constexpr uint32_t kErrPlan = 4u;
inline int quotient_bucket(uint32_t N, bool small) {
    int b = 0;
    while ((N >> (b + 1)) != 0 && b < 15) b++;
    return 2 * b + (small ? 1 : 0);
}
// Frees the ctx's grow-only Karger-Stein scratch (cac_ctx_destroy).
void ctx_scratch_free(cac_ctx *ctx);
// All trials of all queries through one engine, admitted as memory allows.
int mincut_run_queries(cac_ctx *ctx, std::vector<MincutQuery> &queries, float *device_ms);
int mincut_trials(cac_ctx *ctx, const cac_graph *g, uint32_t seed, uint32_t ranks, uint32_t per_rank,
                  uint64_t *d_cuts, float *device_ms);
int ks_dense_one(cac_ctx *ctx, uint32_t n, const uint64_t *mat_host, uint32_t seed, uint32_t rank, uint32_t trial,
                 uint64_t *cut);
int exact_small(cac_ctx *ctx, uint32_t n, const uint64_t *mat_host, uint64_t *cut);

// ---- approx cut (approx.cu) ----
// ref_stream: the reference's own draws (seed replay; unit weights only).
int approx_run(cac_ctx *ctx, const cac_graph *g, double p, uint32_t seed, uint32_t ranks, bool ref_stream,
               cac_approx_result *res);

// ---- sitmo (sitmo_kernels.cu) ----
int sitmo_blocks(cac_ctx *ctx, const uint64_t key[4], const uint64_t ctr0[4], uint64_t nblocks, uint64_t *out_host);

// ---- trial budget (host math shared with the CLI; restated from the reference) ----
uint32_t intermediate_size(uint32_t n, uint64_t m);
uint32_t number_of_trials(uint32_t n, uint64_t m, double p);
uint32_t ks_number_of_trials(uint32_t n, double p);
uint32_t group_draws(uint32_t n);  // the group variant's Stage 1 draws per round
// largest contracted graph the Karger-Stein engine holds as a dense matrix (its contraction
// union-find lives in shared memory)
constexpr uint32_t kMaxDenseVertices = 16384;
int ks_target(int n);
double min_success_in_one_trial(int n);
uint32_t approx_copies(double p);

}  // namespace cac
