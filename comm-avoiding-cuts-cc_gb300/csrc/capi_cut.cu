// C ABI entry points of the cut queries (square_root, approx_cut) and their kernel-level probes.
#include "cac_internal.h"

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

using namespace cac;

extern "C" {

int cac_mincut_trials(cac_ctx *ctx, const cac_graph *g, uint32_t seed, uint32_t virtual_ranks,
                      uint32_t trials_per_rank, uint64_t *cuts_host) {
    if (!ctx || !g || !cuts_host || virtual_ranks == 0) {
        set_error("cac_mincut_trials: invalid argument");
        return CAC_ERR_INVALID;
    }
    if (g->n < 2) {
        set_error("cac_mincut_trials: a cut needs at least two vertices");
        return CAC_ERR_INVALID;
    }
    CAC_CUDA_TRY(cudaSetDevice(ctx->device));
    const uint64_t total = (uint64_t)virtual_ranks * trials_per_rank;
    if (total == 0) return CAC_OK;
    void *d = nullptr;
    CAC_TRY(stream_alloc(ctx, &d, total * 8));
    float ms = 0;
    int st = mincut_trials(ctx, g, seed, virtual_ranks, trials_per_rank, (uint64_t *)d, &ms);
    if (st == CAC_OK) {
        cudaError_t e = cudaMemcpy(cuts_host, d, total * 8, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); st = CAC_ERR_CUDA; }
    }
    stream_free(ctx, d, total * 8);
    return st;
}

int cac_mincut(cac_ctx *ctx, const cac_graph *g, double p, uint32_t seed, uint32_t virtual_ranks,
               cac_mincut_result *res) {
    if (!ctx || !g || !res || !(p >= 0.0 && p < 1.0)) {
        set_error("cac_mincut: invalid argument (success probability must be in [0, 1))");
        return CAC_ERR_INVALID;
    }
    if (g->n < 2) {
        set_error("cac_mincut: a cut needs at least two vertices");
        return CAC_ERR_INVALID;
    }
    if (virtual_ranks == 0) virtual_ranks = 1;
    CAC_CUDA_TRY(cudaSetDevice(ctx->device));
    *res = cac_mincut_result{};
    // SquareRootCut::lowConcurrency (SquareRootCut.cpp:11-13) picks the variant: ceil(T / p)
    // trials per rank (runLowConcurrencyMaster, .cpp:99-100), or p >= 2T and one trial per group
    // of ranks (participateInGroup, .cpp:188-298)
    TrialLayout L{};
    CAC_TRY(trial_layout("cac_mincut", g->n, g->m, p, virtual_ranks, &L));
    res->trials_per_rank = L.per_rank;
    res->total_trials = L.total;
    res->intermediate = intermediate_size(g->n, g->m);
    res->high_concurrency = L.high ? 1u : 0u;
    const uint64_t n_tr = (uint64_t)res->total_trials;
    uint64_t min_degree = 0;
    CAC_TRY(graph_min_degree(ctx, const_cast<cac_graph *>(g), &min_degree));
    void *d = nullptr;
    CAC_TRY(stream_alloc(ctx, &d, n_tr * 8));
    float ms = 0;
    std::vector<MincutQuery> q{
        MincutQuery{g, seed, virtual_ranks, L.per_rank, static_cast<uint64_t *>(d), 0, L.high ? L.groups : 0}};
    int st = mincut_run_queries(ctx, q, &ms);
    if (st == CAC_OK) {
        std::vector<uint64_t> cuts(n_tr);
        cudaError_t e = cudaMemcpy(cuts.data(), d, n_tr * 8, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); st = CAC_ERR_CUDA; }
        else res->cut = std::min(min_degree, *std::min_element(cuts.begin(), cuts.end()));
    }
    res->device_ms = ms;
    stream_free(ctx, d, n_tr * 8);
    return st;
}

int cac_karger_stein(cac_ctx *ctx, const cac_graph *g, double p, uint32_t seed, cac_mincut_result *res) {
    if (!ctx || !g || !res || !(p >= 0.0 && p < 1.0)) {
        set_error("cac_karger_stein: invalid argument (success probability must be in [0, 1))");
        return CAC_ERR_INVALID;
    }
    if (g->n < 2) {
        set_error("cac_karger_stein: a cut needs at least two vertices");
        return CAC_ERR_INVALID;
    }
    CAC_CUDA_TRY(cudaSetDevice(ctx->device));
    *res = cac_mincut_result{};
    const uint32_t trials = ks_number_of_trials(g->n, p);
    res->trials_per_rank = trials;
    res->total_trials = trials;
    res->intermediate = g->n;
    void *d = nullptr;
    CAC_TRY(stream_alloc(ctx, &d, (uint64_t)trials * 8));
    std::vector<MincutQuery> q{MincutQuery{g, seed, 1, trials, static_cast<uint64_t *>(d), g->n}};
    float ms = 0;
    int st = mincut_run_queries(ctx, q, &ms);
    if (st == CAC_OK) {
        std::vector<uint64_t> cuts(trials);
        cudaError_t e = cudaMemcpy(cuts.data(), d, (uint64_t)trials * 8, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            set_error(cudaGetErrorString(e));
            st = CAC_ERR_CUDA;
        } else {
            res->cut = *std::min_element(cuts.begin(), cuts.end());
        }
    }
    res->device_ms = ms;
    stream_free(ctx, d, (uint64_t)trials * 8);
    return st;
}

int cac_karger_stein_trials(cac_ctx *ctx, const cac_graph *g, uint32_t seed, uint32_t trials, uint64_t *cuts_host) {
    if (!ctx || !g || !cuts_host) {
        set_error("cac_karger_stein_trials: invalid argument");
        return CAC_ERR_INVALID;
    }
    if (g->n < 2) {
        set_error("cac_karger_stein_trials: a cut needs at least two vertices");
        return CAC_ERR_INVALID;
    }
    if (trials == 0) return CAC_OK;
    CAC_CUDA_TRY(cudaSetDevice(ctx->device));
    void *d = nullptr;
    CAC_TRY(stream_alloc(ctx, &d, (uint64_t)trials * 8));
    std::vector<MincutQuery> q{MincutQuery{g, seed, 1, trials, static_cast<uint64_t *>(d), g->n}};
    float ms = 0;
    int st = mincut_run_queries(ctx, q, &ms);
    if (st == CAC_OK) {
        cudaError_t e = cudaMemcpy(cuts_host, d, (uint64_t)trials * 8, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            set_error(cudaGetErrorString(e));
            st = CAC_ERR_CUDA;
        }
    }
    stream_free(ctx, d, (uint64_t)trials * 8);
    return st;
}

int cac_mincut_group_trials(cac_ctx *ctx, const cac_graph *g, uint32_t seed, uint32_t groups, uint64_t *cuts_host) {
    if (!ctx || !g || !cuts_host) {
        set_error("cac_mincut_group_trials: invalid argument");
        return CAC_ERR_INVALID;
    }
    if (g->n < 2) {
        set_error("cac_mincut_group_trials: a cut needs at least two vertices");
        return CAC_ERR_INVALID;
    }
    if (groups == 0) return CAC_OK;
    CAC_CUDA_TRY(cudaSetDevice(ctx->device));
    void *d = nullptr;
    CAC_TRY(stream_alloc(ctx, &d, (uint64_t)groups * 8));
    std::vector<MincutQuery> q{MincutQuery{g, seed, groups, 1, static_cast<uint64_t *>(d), 0, groups}};
    float ms = 0;
    int st = mincut_run_queries(ctx, q, &ms);
    if (st == CAC_OK) {
        cudaError_t e = cudaMemcpy(cuts_host, d, (uint64_t)groups * 8, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            set_error(cudaGetErrorString(e));
            st = CAC_ERR_CUDA;
        }
    }
    stream_free(ctx, d, (uint64_t)groups * 8);
    return st;
}

int cac_mincut_batch(cac_ctx *ctx, const cac_mincut_query *queries, uint32_t count, cac_mincut_result *results) {
    if (!ctx || (count && (!queries || !results))) {
        set_error("cac_mincut_batch: invalid argument");
        return CAC_ERR_INVALID;
    }
    CAC_CUDA_TRY(cudaSetDevice(ctx->device));
    std::vector<MincutQuery> qs(count);
    uint64_t total = 0;
    for (uint32_t i = 0; i < count; i++) {
        const cac_mincut_query &q = queries[i];
        if (!q.graph || !(q.success_probability >= 0.0 && q.success_probability < 1.0)) {
            set_error("cac_mincut_batch: query " + std::to_string(i) + " is invalid");
            return CAC_ERR_INVALID;
        }
        if (q.graph->n < 2) {
            set_error("cac_mincut_batch: query " + std::to_string(i) + " has fewer than two vertices");
            return CAC_ERR_INVALID;
        }
        const uint32_t ranks = q.virtual_ranks ? q.virtual_ranks : 1;
        TrialLayout L{};
        CAC_TRY(trial_layout("cac_mincut_batch", q.graph->n, q.graph->m, q.success_probability, ranks, &L));
        results[i] = cac_mincut_result{};
        results[i].trials_per_rank = L.per_rank;
        results[i].total_trials = L.total;
        results[i].intermediate = intermediate_size(q.graph->n, q.graph->m);
        results[i].high_concurrency = L.high ? 1u : 0u;
        qs[i] = MincutQuery{q.graph, q.seed, ranks, L.per_rank, nullptr, 0, L.high ? L.groups : 0};
        total += L.total;
    }
    if (total == 0) return CAC_OK;
    std::vector<uint64_t> min_degree(count);
    for (uint32_t i = 0; i < count; i++)
        CAC_TRY(graph_min_degree(ctx, const_cast<cac_graph *>(queries[i].graph), &min_degree[i]));
    void *d = nullptr;
    CAC_TRY(stream_alloc(ctx, &d, total * 8));
    uint64_t off = 0;
    for (auto &q : qs) {
        q.d_cuts = static_cast<uint64_t *>(d) + off;
        off += q.groups ? (uint64_t)q.groups : (uint64_t)q.ranks * q.per_rank;
    }
    float ms = 0;
    int st = mincut_run_queries(ctx, qs, &ms);
    if (st == CAC_OK) {
        std::vector<uint64_t> cuts(total);
        cudaError_t e = cudaMemcpy(cuts.data(), d, total * 8, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            set_error(cudaGetErrorString(e));
            st = CAC_ERR_CUDA;
        } else {
            off = 0;
            for (uint32_t i = 0; i < count; i++) {
                const uint64_t t = results[i].total_trials;
                results[i].cut = t ? std::min(min_degree[i], *std::min_element(cuts.begin() + off,
                                                                                   cuts.begin() + off + t))
                                   : 0;
                results[i].device_ms = ms;
                off += t;
            }
        }
    }
    stream_free(ctx, d, total * 8);
    return st;
}

int cac_ks_dense(cac_ctx *ctx, uint32_t n, const uint64_t *mat_host, uint32_t seed, uint32_t rank, uint32_t trial,
                 uint64_t *cut) {
    if (!ctx || !mat_host || !cut || n < 2) {
        set_error("cac_ks_dense: invalid argument");
        return CAC_ERR_INVALID;
    }
    CAC_CUDA_TRY(cudaSetDevice(ctx->device));
    return ks_dense_one(ctx, n, mat_host, seed, rank, trial, cut);
}

int cac_exact_cut_small(cac_ctx *ctx, uint32_t n, const uint64_t *mat_host, uint64_t *cut) {
    if (!ctx || !mat_host || !cut || n < 2 || n > 128) {
        set_error("cac_exact_cut_small: invalid argument (2 <= n <= 128)");
        return CAC_ERR_INVALID;
    }
    CAC_CUDA_TRY(cudaSetDevice(ctx->device));
    return exact_small(ctx, n, mat_host, cut);
}

int cac_approx_cut(cac_ctx *ctx, const cac_graph *g, double p, uint32_t seed, uint32_t virtual_ranks,
                   cac_approx_result *res) {
    if (!ctx || !g || !res || !(p > 0.0 && p < 1.0)) {
        set_error("cac_approx_cut: invalid argument (success probability must be in (0, 1))");
        return CAC_ERR_INVALID;
    }
    if (virtual_ranks == 0) virtual_ranks = 1;
    CAC_CUDA_TRY(cudaSetDevice(ctx->device));
    return approx_run(ctx, g, p, seed, virtual_ranks, false, res);
}

int cac_approx_cut_seed_replay(cac_ctx *ctx, const cac_graph *g, double p, uint32_t seed, uint32_t virtual_ranks,
                               cac_approx_result *res) {
    if (!ctx || !g || !res || !(p > 0.0 && p < 1.0)) {
        set_error("cac_approx_cut_seed_replay: invalid argument (success probability must be in (0, 1))");
        return CAC_ERR_INVALID;
    }
    if (virtual_ranks == 0) virtual_ranks = 1;
    CAC_CUDA_TRY(cudaSetDevice(ctx->device));
    return approx_run(ctx, g, p, seed, virtual_ranks, true, res);
}

}  // extern "C"
