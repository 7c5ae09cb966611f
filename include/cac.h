/*
 * cac.h — C ABI of libcac, the GB300 engine for randomized minimum cuts and connected
 * components (drop-in for the square_root / approx_cut / parallel_cc executables of
 * PJK/comm-avoiding-cuts-cc).
 *
 * The reference has no library or FFI interface; its boundary is three command lines, the
 * edge-list file format and one CSV line on stdout. The entry points below replace the
 * callable C++ classes behind those command lines (file:line in the reference tree):
 *
 *   cac_graph_load_file   GraphInputIterator + AdjacencyListGraph::fromIterator
 *                         (src/input/GraphInputIterator.hpp:9-97, src/AdjacencyListGraph.hpp:76-82)
 *   cac_graph_from_edges  AdjacencyListGraph(vertex_count, edges) (src/AdjacencyListGraph.hpp:85-90)
 *   cac_cc                UnweightedIteratedSparseSampling::connectedComponents
 *                         (src/UnweightedIteratedSparseSampling.hpp:19, .cpp:40-72), driven as in
 *                         src/executables/parallel_cc.cpp:28-44
 *   cac_mincut            SquareRootCut::runMaster (src/SquareRootCut.hpp:84, .cpp:15-25),
 *                         driven as in src/executables/square_root.cpp:22-40
 *   cac_mincut_trials     the per-rank trial loop of SquareRootCut::runLowConcurrencyMaster
 *                         (src/SquareRootCut.cpp:127-138), one value per trial
 *   cac_mincut_group_trials  one trial of SquareRootCut::participateInGroup
 *                         (src/SquareRootCut.cpp:188-298) per group, one value per group
 *   cac_ks_dense          comincut::minimum_cut on a dense graph (src/karger-stein/co_mincut.h:491-497)
 *                         for one counter-addressed trial
 *   cac_exact_cut         comincut::deterministic_minimum_cut (src/karger-stein/co_mincut.h:529-541)
 *   cac_approx_cut        ApproximateCut::run (src/ApproximateCut.hpp:62, .cpp:10-79), driven as in
 *                         src/executables/approx_cut.cpp:17-38
 *   cac_sitmo_blocks      sitmo::prng_engine block function (lib/prng_engine.hpp:307-343)
 *   cac_karger_stein      comincut::minimum_cut as src/executables/karger_stein.cpp:34 calls it
 *   cac_cache_write/_convert  a binary form of the edge-list file (no reference counterpart)
 *
 * Conventions
 *   - Every function returns an int status: CAC_OK (0) or a negative CAC_ERR_* code. The
 *     reference throws or asserts instead (SquareRootCut.cpp:44, GraphInputIterator.hpp:19);
 *     cac_last_error() gives the message of the calling thread's last failure.
 *   - Buffers are owned by the caller. Arguments named *_host are host pointers; arguments with
 *     a `where` flag may be host (CAC_HOST) or device (CAC_DEVICE) pointers.
 *   - A cac_ctx binds one device and one CUDA stream; use one ctx per host thread (a ctx is not
 *     thread-safe). All work of a ctx is ordered on its stream; results returned in host
 *     structs are complete when the call returns.
 *   - Vertex ids are uint32 in [0, n); weights uint32 >= 1 (a NULL weight array means 1);
 *     cut values are uint64 sums.
 *   - `virtual_ranks` is the MPI rank count the reference would have run with (mpiexec -n);
 *     it fixes the seed layout (rank r draws with seed + r) and the trial split, not the
 *     hardware parallelism.
 */
#ifndef CAC_H
#define CAC_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CAC_OK 0
#define CAC_ERR_INVALID (-1)     /* bad argument (sizes, ids, null pointers) */
#define CAC_ERR_OOM (-2)         /* device allocation failed or HBM budget exceeded */
#define CAC_ERR_PARSE (-3)       /* malformed edge-list file */
#define CAC_ERR_CUDA (-4)        /* a CUDA runtime call failed */
#define CAC_ERR_TIMEOUT (-5)     /* a device-side bounded wait or draw budget ran out */
#define CAC_ERR_UNSUPPORTED (-6) /* valid request the library does not handle */
#define CAC_ERR_IO (-7)          /* file could not be opened or read */

#define CAC_HOST 0
#define CAC_DEVICE 1

typedef struct cac_ctx cac_ctx;
typedef struct cac_graph cac_graph;

typedef struct {
    int device;                /* CUDA device ordinal */
    void *stream;              /* cudaStream_t to order all work on; NULL: the ctx creates one */
    uint64_t hbm_budget_bytes; /* cap on device bytes this ctx may hold; 0: no cap */
} cac_config;

/* ---- context ---- */
int cac_ctx_create(const cac_config *config, cac_ctx **out);
/* Karger-Stein recursion nodes with more vertices than this (default and maximum 16384, minimum
 * 128), or above 2048 vertices with fewer than N^2 / 32 edges, are kept as edge lists (the
 * reference's sparse recursion, co_mincut.h:401-405); the others as dense matrices. It changes the
 * trials' draws, never the validity of a cut; a lower limit moves more of the recursion to the
 * sparse form. */
int cac_ctx_set_dense_limit(cac_ctx *ctx, uint32_t max_dense_vertices);
/* The quotient kernel of the dense Karger-Stein steps: 0 (default) lets the ctx time the candidates
 * on the first sizeable step of each size bucket and keep the fastest; 1 warp per output row,
 * 2 eight warps per output row, 3 warp per output row with member rows staged by bulk copies, 4 the
 * fixed size rule without timing (eight warps per row from 2000 source vertices on, else one; for
 * profilers, whose serialised replays distort the timings). All give identical matrices; a kernel
 * that does not fit a step's shared memory is replaced by one that does. (No reference
 * counterpart: a tuning control.) */
int cac_ctx_set_quotient_kernel(cac_ctx *ctx, int kind);
/* Karger-Stein levels planned ahead (default 1): every child is taken to stop at its target size,
 * so the levels of a run follow one another without reading the children's sizes back; a child
 * that stops elsewhere (rare: a round that runs out of draws, or a source without edges) is
 * detected on the device and the run is redone level by level. Cuts are identical either way.
 * cac_ctx_plan_redos counts the redone runs. (No reference counterpart: a scheduling control.) */
int cac_ctx_set_plan_ahead(cac_ctx *ctx, int enabled);
uint64_t cac_ctx_plan_redos(const cac_ctx *ctx);
/* Destroys the ctx; graphs still alive are released with it and their handles become invalid. */
int cac_ctx_destroy(cac_ctx *ctx);
const char *cac_error_string(int status);
const char *cac_last_error(void);
/* device bytes currently held by the ctx (graphs + scratch) */
uint64_t cac_ctx_device_bytes(const cac_ctx *ctx);

/* ---- graphs (device-resident) ---- */
int cac_graph_load_file(cac_ctx *ctx, const char *path, cac_graph **out);
int cac_graph_from_edges(cac_ctx *ctx, uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v,
                         const uint32_t *w, int where, cac_graph **out);
int cac_graph_free(cac_graph *g);
/* Copy a graph's edge arrays (m entries each; any pointer may be NULL) to host or device memory. */
int cac_graph_copy_edges(const cac_graph *graph, uint32_t *u, uint32_t *v, uint32_t *w, int where);
int cac_graph_info(const cac_graph *g, uint32_t *n, uint64_t *m, uint64_t *total_weight);
/* Parse an edge-list file into caller-provided host arrays (the file's m must be <= capacity). */
int cac_parse_file(const char *path, uint32_t *n, uint64_t *m, uint32_t *u_host, uint32_t *v_host,
                   uint32_t *w_host, uint64_t capacity);
/* Read only the header (vertex and edge counts) of an edge-list file. */
int cac_parse_header(const char *path, uint32_t *n, uint64_t *m);

/* Binary graph cache: parse a text input once, load it later without parsing (it has no
 * counterpart in the reference). The edge list of a text input is written once; every loader above (cac_graph_load_file, cac_parse_header,
 * cac_parse_file) and every command line accepts the cache file in place of the text file (it is
 * recognised by its magic). Layout, little-endian: "CACG", u32 version 1, u32 n, u32 flags (bit 0:
 * weights stored), u64 m, u64 total weight, then u[m], v[m] and (bit 0) w[m] as u32. Reading
 * checks the length, every endpoint < n and the total weight (CAC_ERR_PARSE otherwise). No GPU
 * is needed for either call. w (nullable) writes an unweighted cache (weights read back as 1). */
int cac_cache_write(const char *path, uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w);
/* Parses a text edge list (all host threads) and writes its cache. */
int cac_cache_convert(const char *input_path, const char *cache_path);

/* ---- connected components (parallel_cc) ---- */
typedef struct {
    uint32_t num_components; /* the count parallel_cc prints */
    uint32_t rounds;         /* sampling rounds + the closing pass over all edges */
    uint64_t sampled_edges;  /* edges drawn in the sampling round */
    float device_ms;         /* device time of the whole call on the ctx stream */
    float edge_pass_ms;      /* device time of the streaming pass over every edge (the loop-dropping
                                filter after a sampling round, else the single hooking pass) */
    float sample_ms;         /* device time of the sampling round (init, draws, compression, bitmap) */
    float hook_ms;           /* device time of hooking the edges that survived the filter */
    float label_ms;          /* device time of the final compression, count and labels */
} cac_cc_result;

/* labels (nullable): label(v) = rank of the smallest vertex of v's component among all
 * component minima, identical to the reference's labels. `labels_where` says whether
 * `labels` is a host or device pointer. */
int cac_cc(cac_ctx *ctx, const cac_graph *g, uint32_t seed, uint32_t virtual_ranks, uint32_t *labels,
           int labels_where, cac_cc_result *res);
/* The same from host edge arrays to host labels in one call (host<->device copies included).
 * Up to 2 Mi edges the edges are copied and the device-resident query runs. Above, the query runs
 * behind the copy: 8 evenly spaced pieces of the list holding the reference's sample budget
 * (n^1.045 * 1.2 edges) cross first and are hooked (res->sampled_edges = their size), then the
 * gaps between them stream through the giant-component filter as they land. Pinned host arrays
 * are faster (the pieces are pulled by a kernel while the gaps are copied); a repeated call with
 * the same arrays replays one captured CUDA graph. The labels are the same either way. The edge
 * arrays are not validated beforehand: an endpoint >= n is skipped by the kernels and the call
 * returns CAC_ERR_INVALID. */
int cac_cc_edges(cac_ctx *ctx, uint32_t n, uint64_t m, const uint32_t *u_host, const uint32_t *v_host,
                 uint32_t seed, uint32_t virtual_ranks, uint32_t *labels_host, cac_cc_result *res);

/* Connected components that allocates nothing. It has no counterpart in the reference. It is for
 * callers that cannot allocate device memory: a plugin inside a host framework whose device
 * memory belongs to that framework's allocator, or a latency-bound serving path that must not
 * take cudaMalloc's implicit synchronisation. The caller passes device inputs and outputs; the
 * scratch is one fixed array of this library that every GPU loading it holds until exit
 * (16 MiB + 33 KiB), so n is limited to 4,194,304 vertices (CAC_ERR_INVALID beyond; cac_cc has no
 * such limit). No ctx is needed: the work is enqueued on `stream` (a cudaStream_t of the current
 * device, NULL for the default stream) and the call returns without synchronising.
 * labels_dev (nullable) gets the same labels as cac_cc; num_components_dev (nullable, device)
 * gets the component count, or 0xFFFFFFFF when an edge endpoint was >= n (such edges are skipped:
 * the edge arrays are not validated beforehand, every endpoint is checked before it is used and
 * the labels are then not valid; with n = 0 and m > 0 every endpoint is out of range, so the count
 * also reads 0xFFFFFFFF). The first call on a device resolves the array's device address
 * (make that first call before any stream capture); if that set-up fails the call returns
 * CAC_ERR_CUDA and a later call retries it. All calls share the one array: calls whose
 * work overlaps on the GPU (other streams, other host threads) race and must be serialised by
 * the caller. */
int cac_cc_noalloc(uint32_t n, uint64_t m, const uint32_t *u_dev, const uint32_t *v_dev, uint32_t *labels_dev,
                   uint32_t *num_components_dev, void *stream);

/* ---- minimum cut (square_root) ---- */
typedef struct {
    uint64_t cut;             /* the CSV `weight` column: the smallest trial value, or the graph's
                                 minimum weighted degree if that is smaller (a single-vertex cut; the
                                 reference reports the trials' minimum alone, so this differs only
                                 when every trial missed a minimum cut around one vertex) */
    uint32_t trials_per_rank; /* the CSV `trials` column: ceil(total / virtual_ranks) */
    uint32_t total_trials;    /* trials executed: virtual_ranks * trials_per_rank, or the group
                                 count in the group variant */
    uint32_t intermediate;    /* t = min(n, ceil(2 sqrt(m) + 1)) */
    uint32_t high_concurrency;/* 1: the group variant ran (virtual_ranks >= 2 * trials, the
                                 reference's SquareRootCut::lowConcurrency, .cpp:11-13): the
                                 ranks form groups of the largest power of two not above
                                 virtual_ranks / trials, each group one trial, trials_per_rank 1 */
    float device_ms;
} cac_mincut_result;

int cac_mincut(cac_ctx *ctx, const cac_graph *g, double success_probability, uint32_t seed,
               uint32_t virtual_ranks, cac_mincut_result *res);
/* Many square_root queries (graphs of any sizes) in one batch: every trial of every query runs
 * through one level-synchronous Karger-Stein engine, admitted as device memory allows. results[i]
 * is what cac_mincut would return for queries[i] alone (device_ms is the whole batch's time).
 * Replaces a loop of SquareRootCut::runMaster calls, one per input graph. */
typedef struct {
    const cac_graph *graph;
    double success_probability;
    uint32_t seed;
    uint32_t virtual_ranks;
} cac_mincut_query;
int cac_mincut_batch(cac_ctx *ctx, const cac_mincut_query *queries, uint32_t count, cac_mincut_result *results);
/* Plain Karger-Stein on the whole graph, as the reference's karger_stein executable runs
 * comincut::minimum_cut (src/executables/karger_stein.cpp, co_mincut.h:515-521): the Karger-Stein
 * library's own trial count for n vertices (comincut::number_of_trials, co_mincut.cpp:44-73), each
 * trial a recursion from the whole graph (no sqrt(m) pre-contraction): its dense matrix, or its edge
 * list when the graph is sparse (above the dense limit, or fewer than n^2 / 32 edges above 2048
 * vertices: the reference's switch, co_mincut.h:401-405); trial i draws from key
 * (seed, i, 1 + heap index).
 * res->trials_per_rank = res->total_trials = the trial count; res->intermediate = n. */
int cac_karger_stein(cac_ctx *ctx, const cac_graph *g, double success_probability, uint32_t seed,
                     cac_mincut_result *res);
/* Run trials (r, i) for r < virtual_ranks, i < trials_per_rank and write each trial's cut to
 * cuts_host[r * trials_per_rank + i]. */
int cac_mincut_trials(cac_ctx *ctx, const cac_graph *g, uint32_t seed, uint32_t virtual_ranks,
                      uint32_t trials_per_rank, uint64_t *cuts_host);
/* Trials 0 .. trials - 1 of plain Karger-Stein (cac_karger_stein's recursion from the whole graph),
 * each trial's cut to cuts_host[i]: the loop of comincut::minimum_cut_trials (co_mincut.h:315-342)
 * with every trial's value kept. */
int cac_karger_stein_trials(cac_ctx *ctx, const cac_graph *g, uint32_t seed, uint32_t trials, uint64_t *cuts_host);
/* Group trials 0 .. groups - 1 of the group variant, each group's cut to cuts_host[g]: Stage 1
 * contracts to t vertices in rounds of floor(n^1.05) weighted draws
 * (WeightedIteratedSparseSampling, .hpp:66-67) with key (seed + g, 0, 1, 0), and two Karger-Stein
 * recursions from the contracted graph (recursive_contract.cpp:45-83 with two trials) take
 * keys (seed + g, 0 | 1, 1 + level, 0); the group's value is the smaller. */
int cac_mincut_group_trials(cac_ctx *ctx, const cac_graph *g, uint32_t seed, uint32_t groups, uint64_t *cuts_host);
/* One Karger-Stein trial (virtual rank, trial index) on a dense symmetric n x n host matrix. */
int cac_ks_dense(cac_ctx *ctx, uint32_t n, const uint64_t *mat_host, uint32_t seed, uint32_t rank, uint32_t trial,
                 uint64_t *cut);
/* Exact minimum cut of a dense symmetric n x n host matrix with n <= 128, computed by the
 * device Stoer-Wagner kernel that solves the Karger-Stein leaves
 * (src/karger-stein/co_mincut_base_case.hpp:52-144 in the reference). */
int cac_exact_cut_small(cac_ctx *ctx, uint32_t n, const uint64_t *mat_host, uint64_t *cut);

/* ---- approximate cut (approx_cut) ---- */
typedef struct {
    uint64_t cut;       /* the CSV `weight` column: 2^level */
    uint32_t trials;    /* the CSV `trials` column: copies * level */
    uint32_t copies;    /* ceil(ln(1-p) / ln(1-e^-0.75)) */
    uint32_t level;     /* first level with more than `copies` components (0: none) */
    float device_ms;
} cac_approx_result;

int cac_approx_cut(cac_ctx *ctx, const cac_graph *g, double success_probability, uint32_t seed,
                   uint32_t virtual_ranks, cac_approx_result *res);

/* approx_cut on the reference's own random draws (seed replay): virtual rank r reads
 * sitmo::prng_engine(seed + r) in the reference's order through std::binomial_distribution<int>
 * as libstdc++ (GCC 13) implements it (ApproximateCut.cpp:33-58), so the answer is the one the
 * reference's approx_cut prints under `mpiexec -n virtual_ranks` with the same seed, where that
 * run is defined. Every edge weight must be 1 (CAC_ERR_UNSUPPORTED otherwise: a weighted edge
 * draws a variable number of outputs, which chains the draws of a rank). Both entry points run
 * min over ranks of ceil(ln w_r) levels, w_r the weight of rank r's slice (the reference's
 * local `w`, ApproximateCut.cpp:19-30). */
int cac_approx_cut_seed_replay(cac_ctx *ctx, const cac_graph *g, double success_probability, uint32_t seed,
                               uint32_t virtual_ranks, cac_approx_result *res);

/* ---- synthetic graphs generated on the device ----
 * Replaces the reference's external generators (utils/generate.py:10-32, er_generator.cpp,
 * sw_generator.cpp, input_generators/rmat_driver.sh:13-16) for the benchmark families. The edge
 * list (order included) and the weights are identical to graphgen.py's host generators for the
 * same arguments. Weights are uniform integers in [wmin, wmax]; the G(n, p) and R-MAT families
 * are unweighted (all 1) when wmax == 1. */
#define CAC_GEN_ERDOS_RENYI 1   /* G(n, p): n, p */
#define CAC_GEN_ERDOS_RENYI_M 2 /* G(n, M), M = floor(n * avg_degree / 2) draws, self-loops dropped: n, avg_degree */
#define CAC_GEN_WATTS_STROGATZ 3 /* ring lattice of k neighbours (k even), rewired with probability p: n, k, p */
#define CAC_GEN_RMAT 4          /* 2^scale vertices, edge_factor * 2^scale edges, quadrants a, b, c, 1-a-b-c */
#define CAC_GEN_COMPLETE 5      /* K_n: n */
typedef struct {
    int family;
    uint32_t n;
    double p;
    double avg_degree;
    uint32_t k;
    uint32_t scale;
    uint32_t edge_factor;
    double a, b, c;
    uint32_t seed;
    uint32_t wmin, wmax;
} cac_gen_spec;
int cac_graph_generate(cac_ctx *ctx, const cac_gen_spec *spec, cac_graph **out);

/* ---- CLICK: the reference's in-memory test graph ----
 * The graph that `square_root|approx_cut PROB CLICK SIZE SEED` builds: the reference's
 * CLICK::generateSlice (src/input/CLICK.hpp:10-49) on every virtual rank r with seed + r, as
 * ApproximateCut::loadFromCLICK does (ApproximateCut.hpp:35, :70-82). K_n in 10 clusters; rank r's
 * enumeration slice gets weights max(0, N(8,4)) (same cluster) or max(0, N(4,4)) from
 * std::mt19937(seed + r), truncated; the E mod P leftover edges belong to no rank, as in the
 * reference. Host code: cac_click_edges needs no device (u == NULL returns the edge count in *m;
 * the arrays must hold it). */
int cac_click_edges(uint32_t n, uint32_t virtual_ranks, uint32_t seed, uint32_t *u, uint32_t *v, uint32_t *w,
                    uint64_t capacity, uint64_t *m);
int cac_graph_click(cac_ctx *ctx, uint32_t n, uint32_t virtual_ranks, uint32_t seed, cac_graph **out);

/* ---- serving loop ----
 * The reference answers one query per process launch. A cac_server keeps graphs resident in HBM
 * and answers square_root, approx_cut and parallel_cc queries as they arrive:
 *   - square_root queries join one persistent Karger-Stein engine between its level steps
 *     (continuous batching: a query admitted while others run shares their launches), admitted
 *     while the estimated footprint of the running queries stays within hbm_budget_bytes
 *     (0: no limit);
 *   - parallel_cc and approx_cut queries run on a second worker and stream, concurrently.
 * The Karger-Stein engine's device buffers count against hbm_budget_bytes: a query whose matrices
 * cannot fit fails alone with CAC_ERR_OOM (a failure inside a shared engine step ends every query
 * running in it with that step's error).
 * Every response equals what the single-query entry point returns for the same arguments
 * (cac_mincut cut and trials_per_rank, cac_approx_cut cut and trials, cac_cc count and labels).
 * Submit and poll may be called from any threads. A graph must outlive the queries on it. */
typedef struct cac_server cac_server;
typedef struct {
    int device;
    uint64_t hbm_budget_bytes;
} cac_server_config;

#define CAC_QUERY_MINCUT 1 /* square_root */
#define CAC_QUERY_APPROX 2 /* approx_cut */
#define CAC_QUERY_CC 3     /* parallel_cc */
#define CAC_PENDING 1      /* cac_server_poll: not finished yet */

typedef struct {
    int kind;                   /* CAC_QUERY_* */
    const cac_graph *graph;     /* from cac_server_graph */
    double success_probability; /* square_root, approx_cut */
    uint32_t seed;
    uint32_t virtual_ranks;     /* 0 is read as 1 */
    uint32_t *labels_host;      /* parallel_cc, optional: n labels written before completion */
} cac_request;

typedef struct {
    int status;              /* CAC_OK or the query's CAC_ERR_* code */
    uint64_t cut;            /* square_root and approx_cut weight */
    uint32_t trials;         /* square_root trials per rank; approx_cut copies * level */
    uint32_t num_components; /* parallel_cc */
    double queue_ms;         /* submit -> admitted */
    double service_ms;       /* admitted -> finished */
    char message[160];       /* the error message when status != CAC_OK */
} cac_response;

int cac_server_create(const cac_server_config *config, cac_server **out);
/* Upload a graph for the server's queries (same arguments as cac_graph_from_edges with host
 * arrays); free it with cac_graph_free after its last query has finished. */
int cac_server_graph(cac_server *server, uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v,
                     const uint32_t *w, cac_graph **out);
/* A generated graph (cac_graph_generate) for the server's queries. */
int cac_server_generate(cac_server *server, const cac_gen_spec *spec, cac_graph **out);
int cac_server_submit(cac_server *server, const cac_request *request, uint64_t *ticket);
/* CAC_OK with *response filled (the ticket is then retired), CAC_PENDING when wait == 0 and the
 * query has not finished, CAC_ERR_INVALID for an unknown ticket. */
int cac_server_poll(cac_server *server, uint64_t ticket, int wait, cac_response *response);
/* Finishes every submitted query, then stops the workers. */
int cac_server_destroy(cac_server *server);

/* ---- primitives ---- */
/* nblocks sitmo blocks with key `key` and counters ctr0, ctr0 + 1, ... (256-bit add);
 * out_host receives 4 * nblocks uint64 words. */
int cac_sitmo_blocks(cac_ctx *ctx, const uint64_t key[4], const uint64_t ctr0[4], uint64_t nblocks,
                     uint64_t *out_host);

#ifdef __cplusplus
}
#endif

#endif
