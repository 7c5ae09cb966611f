// libcac runtime: contexts, device memory accounting, graphs and the C ABI entry points.
#include "cac_internal.h"

#include <mutex>
#include <set>
#include <utility>
#include "sitmo.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

namespace cac {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int smem_optin(cac_ctx *ctx, const void *func) {
    static std::mutex mu;
    static std::set<std::pair<int, const void *>> raised;
    std::lock_guard<std::mutex> lk(mu);
    if (raised.count({ctx->device, func})) return CAC_OK;
    int optin = 0;
    CAC_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
    cudaFuncAttributes fa{};
    CAC_CUDA_TRY(cudaFuncGetAttributes(&fa, func));
    CAC_CUDA_TRY(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      optin - (int)fa.sharedSizeBytes));
    raised.insert({ctx->device, func});
    return CAC_OK;
}

int dev_alloc(cac_ctx *ctx, void **p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) return CAC_OK;
    if (ctx->budget && ctx->held + bytes > ctx->budget) {
        set_error("HBM budget exceeded: need " + std::to_string(ctx->held + bytes) + " bytes, budget " +
                  std::to_string(ctx->budget));
        return CAC_ERR_OOM;
    }
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        set_error(std::string("cudaMalloc(") + std::to_string(bytes) + "): " + cudaGetErrorString(e));
        return CAC_ERR_OOM;
    }
    ctx->held += bytes;
    return CAC_OK;
}

int stream_alloc(cac_ctx *ctx, void **p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) return CAC_OK;
    if (ctx->budget && ctx->held + bytes > ctx->budget) {
        set_error("HBM budget exceeded: need " + std::to_string(ctx->held + bytes) + " bytes, budget " +
                  std::to_string(ctx->budget));
        return CAC_ERR_OOM;
    }
    cudaError_t e = ctx->pool ? cudaMallocFromPoolAsync(p, bytes, ctx->pool, ctx->stream)
                              : cudaMallocAsync(p, bytes, ctx->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        set_error(std::string("cudaMallocAsync(") + std::to_string(bytes) + "): " + cudaGetErrorString(e));
        return CAC_ERR_OOM;
    }
    ctx->held += bytes;
    return CAC_OK;
}

void stream_free(cac_ctx *ctx, void *p, size_t bytes) {
    if (!p) return;
    if (cudaFreeAsync(p, ctx->stream) != cudaSuccess) {
        const cudaError_t e = cudaGetLastError();
        set_error(std::string("cudaFreeAsync: ") + cudaGetErrorString(e));
    }
    ctx->held -= std::min<uint64_t>(ctx->held, bytes);
}

void dev_free(cac_ctx *ctx, void *p, size_t bytes) {
    if (!p) return;
    if (cudaFree(p) != cudaSuccess) {
        const cudaError_t e = cudaGetLastError();  // not left behind as a sticky error for an unrelated check
        set_error(std::string("cudaFree: ") + cudaGetErrorString(e));
    }
    ctx->held -= std::min<uint64_t>(ctx->held, bytes);
}

int arena_reserve(cac_ctx *ctx, Arena &a, size_t bytes) {
    if (bytes <= a.cap) return CAC_OK;
    CAC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    dev_free(ctx, a.base, a.cap);
    a.base = nullptr;
    a.cap = 0;
    a.used = 0;
    size_t want = align_up(bytes, 1 << 20);
    void *p = nullptr;
    CAC_TRY(dev_alloc(ctx, &p, want));
    a.base = (char *)p;
    a.cap = want;
    return CAC_OK;
}

void *arena_take(Arena &a, size_t bytes) {
    size_t at = align_up(a.used);
    a.used = at + align_up(bytes);
    return a.base + at;
}

// ---- trial budget: the reference's double-precision expressions ----

int ks_target(int n) {
    // comincut::target_number_of_vertices_for_contraction (co_mincut.cpp:18-20)
    int t = (int)std::ceil((double)n / std::sqrt((double)2)) + 1;
    return std::max(t, 128);
}

double min_success_in_one_trial(int n) {
    // comincut::min_success_in_one_trial (co_mincut.cpp:32-41)
    if (n <= 128) return 1;
    double r = min_success_in_one_trial(ks_target(n));
    return 1.0 - std::pow((1 - 0.5 * r), 2);
}

uint32_t intermediate_size(uint32_t n, uint64_t m) {
    // SquareRootCut::intermediate_size (SquareRootCut.cpp:63-70), base_case_multiplier = 2
    uint32_t c = (uint32_t)std::ceil(2.0 * std::sqrt((double)m) + 1);
    return c > n ? n : c;
}

uint32_t number_of_trials(uint32_t n, uint64_t m, double p) {
    // SquareRootCut::numberOfTrials (SquareRootCut.cpp:76-83)
    double pk = min_success_in_one_trial((int)intermediate_size(n, m));
    double c = 1.0 / (1 - p);
    return (uint32_t)std::ceil(((double)n * ((double)n * std::log(c))) / (2.0 * 2.0 * ((double)m * pk)));
}

int trial_layout(const char *who, uint32_t n, uint64_t m, double p, uint32_t ranks, TrialLayout *out) {
    if (ranks == 0) ranks = 1;
    const uint32_t total = number_of_trials(n, m, p);
    TrialLayout L{};
    L.high = (double)ranks >= 2.0 * total;
    if (L.high) {
        // participateInGroup: processors_per_trial = p / T (integer), group_size the largest power
        // of two not above it, group_count = p / group_size
        const uint32_t per = total ? ranks / total : ranks;
        uint32_t size = 1;
        while ((uint64_t)size * 2 <= per) size *= 2;
        L.groups = ranks / size;
        L.per_rank = 1;
        L.total = L.groups;
    } else {
        const uint64_t per = (uint64_t)std::ceil((double)total / ranks);
        const uint64_t all = per * ranks;
        if (per > 0xFFFFFFFFull || all > 0xFFFFFFFFull) {
            set_error(std::string(who) + ": " + std::to_string(all) + " trials (" + std::to_string(ranks) +
                      " virtual ranks) exceed 2^32 - 1");
            return CAC_ERR_INVALID;
        }
        L.per_rank = (uint32_t)per;
        L.total = (uint32_t)all;
    }
    *out = L;
    return CAC_OK;
}

uint32_t group_draws(uint32_t n) {
    // edgesToSamplePerProcessor (WeightedIteratedSparseSampling.hpp:66-67): floor(n0^(1 + 0.1 / 2)) in float
    return (uint32_t)std::pow((float)n, 1.0f + 0.1f / 2.0f);
}

uint32_t ks_number_of_trials(uint32_t n, double p) {
    // comincut::number_of_trials (co_mincut.cpp:44-73): multiply the failure probability of one
    // trial until it is at most 1 - p
    if (n <= 128 || p == 0) return 1;
    const double one = min_success_in_one_trial((int)n);
    double failure = 1.0;
    uint32_t trials = 0;
    while (failure > 1.0 - p) {
        failure *= 1.0 - one;
        trials++;
    }
    return trials;
}

uint32_t approx_copies(double p) {
    // ApproximateCut::numberOfTrials (ApproximateCut.cpp:82-87)
    double alpha = std::log(1 - std::exp(-(double)0.75));
    return (uint32_t)std::ceil(std::log((double)1.0 - p) / alpha);
}

namespace {

__global__ void fill_u32(uint32_t *p, uint64_t n, uint32_t value) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = value;
}

// Total of the weights, and a flag set when any weight is not 1.
__global__ void sum_u32(const uint32_t *p, uint64_t n, unsigned long long *out, unsigned int *nonunit) {
    uint64_t acc = 0;
    uint32_t odd = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        acc += p[i];
        odd |= p[i] != 1u;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    odd = __any_sync(0xffffffffu, odd);
    if ((threadIdx.x & 31) == 0) {
        if (acc) atomicAdd(out, (unsigned long long)acc);
        if (odd) atomicOr(nonunit, 1u);
    }
}

__global__ void check_ids(const uint32_t *u, const uint32_t *v, uint64_t m, uint32_t n, unsigned int *bad) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x)
        if (u[i] >= n || v[i] >= n) atomicOr(bad, 1u);
}

__global__ void sitmo_blocks_kernel(uint64_t k0, uint64_t k1, uint64_t k2, uint64_t k3, uint64_t c0, uint64_t c1,
                                    uint64_t c2, uint64_t c3, uint64_t nblocks, uint64_t *out) {
    for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nblocks;
         b += (uint64_t)gridDim.x * blockDim.x) {
        // 256-bit counter ctr0 + b
        uint64_t d0 = c0 + b, carry = d0 < c0;
        uint64_t d1 = c1 + carry;
        carry = carry && d1 == 0;
        uint64_t d2 = c2 + carry;
        carry = carry && d2 == 0;
        uint64_t d3 = c3 + carry;
        u64x4 o = sitmo_block(k0, k1, k2, k3, d0, d1, d2, d3);
        for (int j = 0; j < 4; j++) out[4 * b + j] = o.x[j];
    }
}

// Weighted degree of every vertex (loops skipped), one u64 atomic per endpoint.
__global__ void degree_add(const uint32_t *u, const uint32_t *v, const uint32_t *w, uint64_t m,
                           unsigned long long *deg) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t a = u[e], b = v[e];
        if (a == b) continue;
        atomicAdd(deg + a, (unsigned long long)w[e]);
        atomicAdd(deg + b, (unsigned long long)w[e]);
    }
}

// Minimum over n degrees: a warp minimum, then one atomicMin per warp.
__global__ void degree_min(const unsigned long long *deg, uint32_t n, unsigned long long *out) {
    unsigned long long x = ~0ull;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        x = min(x, deg[i]);
    for (int o = 16; o > 0; o >>= 1) x = min(x, __shfl_xor_sync(0xffffffffu, x, o));
    if ((threadIdx.x & 31) == 0) atomicMin(out, x);
}

int grid1(cac_ctx *ctx, uint64_t work) {
    uint64_t need = (work + 255) / 256;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(need, (uint64_t)ctx->num_sms * 8));
}

}  // namespace

int sitmo_blocks(cac_ctx *ctx, const uint64_t key[4], const uint64_t ctr0[4], uint64_t nblocks, uint64_t *out_host) {
    if (nblocks == 0) return CAC_OK;
    CAC_TRY(arena_reserve(ctx, nblocks * 32));
    arena_reset(ctx);
    uint64_t *d = (uint64_t *)arena_take(ctx, nblocks * 32);
    sitmo_blocks_kernel<<<grid1(ctx, nblocks), 256, 0, ctx->stream>>>(key[0], key[1], key[2], key[3], ctr0[0],
                                                                      ctr0[1], ctr0[2], ctr0[3], nblocks, d);
    CAC_CUDA_TRY(cudaGetLastError());
    CAC_CUDA_TRY(cudaMemcpyAsync(out_host, d, nblocks * 32, cudaMemcpyDeviceToHost, ctx->stream));
    CAC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return CAC_OK;
}

int graph_min_degree(cac_ctx *ctx, cac_graph *g, uint64_t *out) {
    static std::mutex mu;  // graphs may be shared by the threads of a server
    std::lock_guard<std::mutex> lock(mu);
    if (!g->min_degree_known) {
        void *d = nullptr;
        const size_t bytes = ((size_t)g->n + 1) * 8;
        CAC_TRY(stream_alloc(ctx, &d, bytes));
        unsigned long long *deg = static_cast<unsigned long long *>(d), *res = deg + g->n;
        cudaStream_t s = ctx->stream;
        unsigned long long h = 0;
        cudaError_t e = cudaMemsetAsync(deg, 0, (size_t)g->n * 8, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(res, 0xFF, 8, s);
        if (e == cudaSuccess && g->m) {
            degree_add<<<grid1(ctx, g->m), 256, 0, s>>>(g->u, g->v, g->w, g->m, deg);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) {
            degree_min<<<grid1(ctx, g->n), 256, 0, s>>>(deg, g->n, res);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(&h, res, 8, cudaMemcpyDeviceToHost, s);
        stream_free(ctx, d, bytes);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error(std::string("minimum weighted degree: ") + cudaGetErrorString(e));
            return CAC_ERR_CUDA;
        }
        g->min_degree = h;
        g->min_degree_known = true;
    }
    *out = g->min_degree;
    return CAC_OK;
}

int graph_create(cac_ctx *ctx, uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w,
                 int where, cac_graph **out) {
    cac_graph *g = new (std::nothrow) cac_graph();
    if (!g) { set_error("host allocation failed"); return CAC_ERR_OOM; }
    g->ctx = ctx;
    g->n = n;
    g->m = m;
    const size_t b = align_up(m * 4);
    g->bytes = 3 * b;
    void *p = nullptr;
    int st = dev_alloc(ctx, &p, g->bytes ? g->bytes : 256);
    if (st != CAC_OK) { delete g; return st; }
    if (!g->bytes) g->bytes = 256;
    g->u = (uint32_t *)p;
    g->v = (uint32_t *)((char *)p + b);
    g->w = (uint32_t *)((char *)p + 2 * b);
    cudaStream_t s = ctx->stream;
    const cudaMemcpyKind kind = where == CAC_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    auto fail = [&](int code) { dev_free(ctx, p, g->bytes); delete g; return code; };
    if (m) {
        if (cudaMemcpyAsync(g->u, u, m * 4, kind, s) != cudaSuccess ||
            cudaMemcpyAsync(g->v, v, m * 4, kind, s) != cudaSuccess) {
            set_error("edge upload failed");
            return fail(CAC_ERR_CUDA);
        }
        if (w) {
            if (cudaMemcpyAsync(g->w, w, m * 4, kind, s) != cudaSuccess) {
                set_error("weight upload failed");
                return fail(CAC_ERR_CUDA);
            }
        } else {
            fill_u32<<<grid1(ctx, m), 256, 0, s>>>(g->w, m, 1u);
        }
        // validate ids and total the weights on the device
        int st2 = arena_reserve(ctx, 256);
        if (st2 != CAC_OK) return fail(st2);
        arena_reset(ctx);
        unsigned long long *d_sum = (unsigned long long *)arena_take(ctx, 16);
        unsigned int *d_bad = (unsigned int *)(d_sum + 1);
        cudaMemsetAsync(d_sum, 0, 16, s);
        check_ids<<<grid1(ctx, m), 256, 0, s>>>(g->u, g->v, m, n, d_bad);
        sum_u32<<<grid1(ctx, m), 256, 0, s>>>(g->w, m, d_sum, d_bad + 1);
        unsigned long long hsum[2] = {0, 0};
        if (cudaMemcpyAsync(hsum, d_sum, 16, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            set_error(std::string("graph validation failed: ") + cudaGetErrorString(cudaGetLastError()));
            return fail(CAC_ERR_CUDA);
        }
        if ((unsigned int)(hsum[1] & 0xFFFFFFFFu)) {
            set_error("edge endpoint id >= vertex count " + std::to_string(n));
            return fail(CAC_ERR_INVALID);
        }
        g->total_weight = hsum[0];
        g->unit_weights = (hsum[1] >> 32) == 0;
    }
    ctx->graphs.insert(g);
    *out = g;
    return CAC_OK;
}

}  // namespace cac

using namespace cac;

extern "C" {

int cac_ctx_set_dense_limit(cac_ctx *ctx, uint32_t max_dense_vertices) {
    if (!ctx || max_dense_vertices < 128 || max_dense_vertices > kMaxDenseVertices) {
        set_error("cac_ctx_set_dense_limit: the limit must be in [128, 16384]");
        return CAC_ERR_INVALID;
    }
    ctx->dense_limit = max_dense_vertices;
    return CAC_OK;
}

int cac_ctx_set_quotient_kernel(cac_ctx *ctx, int kind) {
    if (!ctx || kind < 0 || kind > 4) {
        set_error("cac_ctx_set_quotient_kernel: kind must be 0 (autotuned), 1, 2, 3 or 4 (the size rule)");
        return CAC_ERR_INVALID;
    }
    ctx->quotient_forced = (uint8_t)kind;
    return CAC_OK;
}

int cac_ctx_set_plan_ahead(cac_ctx *ctx, int enabled) {
    if (!ctx) {
        set_error("cac_ctx_set_plan_ahead: invalid argument");
        return CAC_ERR_INVALID;
    }
    ctx->plan_ahead = enabled != 0;
    return CAC_OK;
}

uint64_t cac_ctx_plan_redos(const cac_ctx *ctx) { return ctx ? ctx->plan_redos : 0; }

const char *cac_error_string(int status) {
    switch (status) {
        case CAC_OK: return "ok";
        case CAC_ERR_INVALID: return "invalid argument";
        case CAC_ERR_OOM: return "out of device memory or HBM budget";
        case CAC_ERR_PARSE: return "malformed edge-list input";
        case CAC_ERR_CUDA: return "CUDA runtime error";
        case CAC_ERR_TIMEOUT: return "device-side bound exceeded";
        case CAC_ERR_UNSUPPORTED: return "unsupported request";
        case CAC_ERR_IO: return "input could not be read";
        default: return "unknown status";
    }
}

const char *cac_last_error(void) { return g_last_error.c_str(); }

int cac_ctx_create(const cac_config *config, cac_ctx **out) {
    if (!out) { set_error("cac_ctx_create: out is NULL"); return CAC_ERR_INVALID; }
    *out = nullptr;
    cac_config cfg{};
    if (config) cfg = *config;
    int ndev = 0;
    CAC_CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (cfg.device < 0 || cfg.device >= ndev) {
        set_error("cac_ctx_create: device " + std::to_string(cfg.device) + " not present");
        return CAC_ERR_INVALID;
    }
    CAC_CUDA_TRY(cudaSetDevice(cfg.device));
    cac_ctx *ctx = new (std::nothrow) cac_ctx();
    if (!ctx) { set_error("host allocation failed"); return CAC_ERR_OOM; }
    ctx->device = cfg.device;
    ctx->budget = cfg.hbm_budget_bytes;
    if (cfg.stream) {
        ctx->stream = (cudaStream_t)cfg.stream;
    } else {
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete ctx;
            set_error("cudaStreamCreate failed");
            return CAC_ERR_CUDA;
        }
        ctx->own_stream = true;
    }
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, cfg.device);
    {
        // a pool of its own for the level buffers, which keeps freed memory for the next level
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = cfg.device;
        if (cudaMemPoolCreate(&ctx->pool, &props) == cudaSuccess) {
            uint64_t keep = ~0ull;
            cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep);
        } else {
            cudaGetLastError();
            ctx->pool = nullptr;
        }
    }
    for (auto &e : ctx->ev) cudaEventCreate(&e);
    if (cudaMallocHost((void **)&ctx->pinned_u32, 64 * 1024) != cudaSuccess) {
        set_error("cudaMallocHost failed");
        cac_ctx_destroy(ctx);
        return CAC_ERR_CUDA;
    }
    *out = ctx;
    return CAC_OK;
}

int cac_ctx_destroy(cac_ctx *ctx) {
    if (!ctx) return CAC_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    // graphs still alive are released with their ctx; their handles become invalid
    for (cac_graph *g : ctx->graphs) {
        dev_free(ctx, g->u, g->bytes);
        delete g;
    }
    ctx->graphs.clear();
    cc_graph_reset(ctx);
    ctx_scratch_free(ctx);
    dev_free(ctx, ctx->arena.base, ctx->arena.cap);
    dev_free(ctx, ctx->io.base, ctx->io.cap);
    if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
    for (auto &e : ctx->ev) if (e) cudaEventDestroy(e);
    for (auto &e : ctx->chunk_ev) if (e) cudaEventDestroy(e);
    if (ctx->copy_stream) {
        cudaStreamSynchronize(ctx->copy_stream);
        cudaStreamDestroy(ctx->copy_stream);
    }
    if (ctx->pinned_u32) cudaFreeHost(ctx->pinned_u32);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return CAC_OK;
}

uint64_t cac_ctx_device_bytes(const cac_ctx *ctx) { return ctx ? ctx->held : 0; }

int cac_graph_from_edges(cac_ctx *ctx, uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v,
                         const uint32_t *w, int where, cac_graph **out) {
    if (!ctx || !out || (m && (!u || !v)) || (where != CAC_HOST && where != CAC_DEVICE)) {
        set_error("cac_graph_from_edges: invalid argument");
        return CAC_ERR_INVALID;
    }
    if (m > 0xFFFFFFFFull) {
        set_error("cac_graph_from_edges: more than 2^32-1 edges (the reference counts edges in unsigned)");
        return CAC_ERR_UNSUPPORTED;
    }
    CAC_CUDA_TRY(cudaSetDevice(ctx->device));
    return graph_create(ctx, n, m, u, v, w, where, out);
}

int cac_graph_free(cac_graph *g) {
    if (!g) return CAC_OK;
    cac_ctx *ctx = g->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    ctx->graphs.erase(g);
    dev_free(ctx, g->u, g->bytes);
    delete g;
    return CAC_OK;
}

int cac_graph_copy_edges(const cac_graph *g, uint32_t *u, uint32_t *v, uint32_t *w, int where) {
    if (!g || (where != CAC_HOST && where != CAC_DEVICE)) {
        set_error("cac_graph_copy_edges: invalid argument");
        return CAC_ERR_INVALID;
    }
    cac_ctx *ctx = g->ctx;
    CAC_CUDA_TRY(cudaSetDevice(ctx->device));
    const cudaMemcpyKind kind = where == CAC_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    const size_t b = g->m * 4;
    if (b) {
        if (u) CAC_CUDA_TRY(cudaMemcpyAsync(u, g->u, b, kind, ctx->stream));
        if (v) CAC_CUDA_TRY(cudaMemcpyAsync(v, g->v, b, kind, ctx->stream));
        if (w) CAC_CUDA_TRY(cudaMemcpyAsync(w, g->w, b, kind, ctx->stream));
    }
    CAC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return CAC_OK;
}

int cac_graph_info(const cac_graph *g, uint32_t *n, uint64_t *m, uint64_t *total_weight) {
    if (!g) { set_error("cac_graph_info: graph is NULL"); return CAC_ERR_INVALID; }
    if (n) *n = g->n;
    if (m) *m = g->m;
    if (total_weight) *total_weight = g->total_weight;
    return CAC_OK;
}

int cac_cc(cac_ctx *ctx, const cac_graph *g, uint32_t seed, uint32_t virtual_ranks, uint32_t *labels,
           int labels_where, cac_cc_result *res) {
    if (!ctx || !g || (labels && labels_where != CAC_HOST && labels_where != CAC_DEVICE)) {
        set_error("cac_cc: invalid argument");
        return CAC_ERR_INVALID;
    }
    CAC_CUDA_TRY(cudaSetDevice(ctx->device));
    if (virtual_ranks == 0) virtual_ranks = 1;
    uint32_t *d_labels = nullptr;
    if (labels && labels_where == CAC_DEVICE) d_labels = labels;
    if (labels && labels_where == CAC_HOST) {
        // device staging for host labels: the ctx's grow-only io arena (a stable address, so a
        // repeated query can replay its captured launch sequence)
        CAC_TRY(arena_reserve(ctx, ctx->io, (size_t)g->n * 4 + 4));
        ctx->io.used = 0;
        d_labels = (uint32_t *)arena_take(ctx->io, (size_t)g->n * 4 + 4);
    }
    cac_cc_result r{};
    int st = cc_run(ctx, g->n, g->m, g->u, g->v, seed, virtual_ranks, d_labels, &r);
    if (st == CAC_OK && labels && labels_where == CAC_HOST && g->n) {
        cudaError_t e = cudaMemcpyAsync(labels, d_labels, (size_t)g->n * 4, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); st = CAC_ERR_CUDA; }
    }
    if (res) *res = r;
    return st;
}

int cac_cc_edges(cac_ctx *ctx, uint32_t n, uint64_t m, const uint32_t *u_host, const uint32_t *v_host,
                 uint32_t seed, uint32_t virtual_ranks, uint32_t *labels_host, cac_cc_result *res) {
    if (!ctx || (m && (!u_host || !v_host))) {
        set_error("cac_cc_edges: invalid argument");
        return CAC_ERR_INVALID;
    }
    CAC_CUDA_TRY(cudaSetDevice(ctx->device));
    if (virtual_ranks == 0) virtual_ranks = 1;
    // staging buffers for edges and labels: a grow-only arena kept by the ctx
    const size_t be = align_up(m * 4), bl = align_up((size_t)n * 4 + 4);
    CAC_TRY(arena_reserve(ctx, ctx->io, 2 * be + bl));
    ctx->io.used = 0;
    uint32_t *du = (uint32_t *)arena_take(ctx->io, m * 4);
    uint32_t *dv = (uint32_t *)arena_take(ctx->io, m * 4);
    uint32_t *dl = (uint32_t *)arena_take(ctx->io, (size_t)n * 4 + 4);
    cudaStream_t s = ctx->stream;
    int st = CAC_OK;
    cac_cc_result r{};
    // Up to 2 Mi edges, copy then run the device-resident query (sampling round + filter). Above,
    // the edges cross in an order that lets the query run behind the copy (cc_run_streamed),
    // measured faster from 4 M edges on (e.g. 0.36 vs 0.41 ms on G(500000, M) with 4 M edges, 0.75
    // vs 0.91 ms on BA n=1,024,000, 2.82 vs 3.35 ms on R-MAT scale 22) and equal at 2 Mi.
    bool streamed = false;
    if (m <= (2ull << 20)) {
        if (m && (cudaMemcpyAsync(du, u_host, m * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
                  cudaMemcpyAsync(dv, v_host, m * 4, cudaMemcpyHostToDevice, s) != cudaSuccess)) {
            set_error("cac_cc_edges: upload failed");
            st = CAC_ERR_CUDA;
        }
        if (st == CAC_OK) st = cc_run(ctx, n, m, du, dv, seed, virtual_ranks, labels_host ? dl : nullptr, &r, true);
    } else {
        st = cc_run_streamed(ctx, n, m, u_host, v_host, du, dv, labels_host ? dl : nullptr, labels_host, &r);
        streamed = true;
    }
    if (st == CAC_OK && labels_host && n && !streamed) {
        if (cudaMemcpyAsync(labels_host, dl, (size_t)n * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            set_error("cac_cc_edges: label download failed");
            st = CAC_ERR_CUDA;
        }
    }
    if (res) *res = r;
    return st;
}

int cac_sitmo_blocks(cac_ctx *ctx, const uint64_t key[4], const uint64_t ctr0[4], uint64_t nblocks,
                     uint64_t *out_host) {
    if (!ctx || !key || !ctr0 || (nblocks && !out_host)) {
        set_error("cac_sitmo_blocks: invalid argument");
        return CAC_ERR_INVALID;
    }
    CAC_CUDA_TRY(cudaSetDevice(ctx->device));
    return sitmo_blocks(ctx, key, ctr0, nblocks, out_host);
}

}  // extern "C"
