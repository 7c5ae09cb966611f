// approx_cut: the GB300 form of ApproximateCut::run (src/ApproximateCut.cpp:10-79).
//
// For levels i = 1 .. ceil(ln W) the reference keeps each edge of each of `copies` disjoint
// copies iff Binomial(w, 2^-i) > 0 (std::binomial_distribution, :39-48), relabels copy j to
// v + j n, runs the iterated-sparse-sampling CC on the union and stops at the first level with
// more than `copies` components; the answer is 2^level.
//
// Here one kernel per level does the keep test of every (copy, edge) pair and hooks kept edges
// straight into one union-find over n * copies vertices (the CC of the disjoint union is the
// union-find of all kept edges; the CC path's sampling round has nothing to skip at these
// densities), then the roots are counted. The keep test is integer-only and counter-addressed:
// P(Binomial(w, q) > 0) = 1 - (1 - q)^w, so the pair is kept iff the u64 draw x >= F(i, w) with
// F = (1 - 2^-i)^w in 0.64 fixed point by square-and-multiply over truncating 64x64->128-bit
// products; x is draw e_local of stream (seed + r, i, j, 1), r the virtual rank whose slice
// holds the edge (ApproximateCut::loadFromInput, ApproximateCut.hpp:64-68) and e_local its
// index in that slice. oracle/approx.c replays the same rule on the host.
#include "cac_internal.h"
#include "sitmo.cuh"

#include <algorithm>
#include <cmath>

namespace cac {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ uint64_t keep_threshold(uint32_t level, uint32_t w) {
    const uint64_t base = 0ull - (1ull << (64 - level));
    uint64_t res = base, b = base;
    uint32_t e = w - 1;
    while (e) {
        if (e & 1) res = mulhi64(res, b);
        b = mulhi64(b, b);
        e >>= 1;
    }
    return res;
}

__device__ __forceinline__ uint32_t afind(uint32_t *par, uint32_t v) {
    uint32_t cur = par[v];
    if (cur != v) {
        uint32_t prev = v, next;
        while (cur > (next = par[cur])) {
            par[prev] = next;
            prev = cur;
            cur = next;
        }
    }
    return cur;
}

__device__ __forceinline__ void aunite(uint32_t *par, uint32_t a, uint32_t b) {
    uint32_t ra = afind(par, a), rb = afind(par, b);
    while (ra != rb) {
        if (ra < rb) {
            const uint32_t old = atomicCAS(&par[rb], rb, ra);
            if (old == rb) return;
            rb = old;
        } else {
            const uint32_t old = atomicCAS(&par[ra], ra, rb);
            if (old == ra) return;
            ra = old;
        }
    }
}

__global__ void approx_init(uint32_t *par, uint64_t nv) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (uint64_t)gridDim.x * blockDim.x)
        par[i] = (uint32_t)i;
}

// One thread per (copy, edge); copies along blockIdx.y.
__global__ void approx_keep_hook(uint32_t *par, const uint32_t *__restrict__ U, const uint32_t *__restrict__ V,
                                 const uint32_t *__restrict__ Wt, uint64_t m, uint32_t n, uint32_t level,
                                 uint32_t seed, uint32_t ranks, uint64_t portion) {
    const uint32_t j = blockIdx.y;
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t w = Wt[e];
        if (w == 0) continue;
        const uint64_t q = portion ? e / portion : (uint64_t)ranks;
        const uint32_t r = q < ranks ? (uint32_t)q : ranks - 1;
        const uint64_t local = e - (uint64_t)r * portion;
        const uint64_t x = draw64(seed + r, level, j, 1, 0, local);
        if (x < keep_threshold(level, w)) continue;
        const uint32_t off = j * n;
        aunite(par, U[e] + off, V[e] + off);
    }
}

__global__ void approx_count_roots(const uint32_t *par, uint64_t nv, unsigned int *count) {
    uint32_t c = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (uint64_t)gridDim.x * blockDim.x)
        c += par[i] == (uint32_t)i;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

}  // namespace

int approx_run(cac_ctx *ctx, const cac_graph *g, double p, uint32_t seed, uint32_t ranks, cac_approx_result *res) {
    cudaStream_t s = ctx->stream;
    *res = cac_approx_result{};
    const uint32_t copies = approx_copies(p);
    res->copies = copies;
    const uint64_t nv = (uint64_t)g->n * copies;
    if (nv >= 0xFFFFFFFFull) {
        set_error("approx_cut: n * copies must stay below 2^32");
        return CAC_ERR_UNSUPPORTED;
    }
    // ApproximateCut.cpp:30: (unsigned) ceil(log(w)); levels beyond 63 cannot occur for 64-bit sums
    const uint32_t iterations = g->total_weight ? (uint32_t)std::ceil(std::log((double)g->total_weight)) : 0;
    CAC_TRY(arena_reserve(ctx, align_up(nv * 4 + 4) + 256));
    arena_reset(ctx);
    uint32_t *par = (uint32_t *)arena_take(ctx, nv * 4 + 4);
    unsigned int *d_count = (unsigned int *)arena_take(ctx, 16);
    const uint64_t portion = g->m / ranks;
    const int gi = (int)std::max<uint64_t>(1, std::min<uint64_t>((nv + kThreads - 1) / kThreads, ctx->num_sms * 8));
    const int ge = (int)std::max<uint64_t>(1, std::min<uint64_t>((g->m + kThreads - 1) / kThreads,
                                                                  std::max(1, ctx->num_sms * 8 / (int)copies)));
    CAC_CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
    uint32_t first = 0;
    for (uint32_t level = 1; level <= iterations && level <= 63; level++) {
        approx_init<<<gi, kThreads, 0, s>>>(par, nv);
        if (g->m) {
            dim3 grid(ge, copies);
            approx_keep_hook<<<grid, kThreads, 0, s>>>(par, g->u, g->v, g->w, g->m, g->n, level, seed, ranks, portion);
        }
        CAC_CUDA_TRY(cudaMemsetAsync(d_count, 0, 4, s));
        approx_count_roots<<<gi, kThreads, 0, s>>>(par, nv, d_count);
        CAC_CUDA_TRY(cudaGetLastError());
        CAC_CUDA_TRY(cudaMemcpyAsync(ctx->pinned_u32, d_count, 4, cudaMemcpyDeviceToHost, s));
        CAC_CUDA_TRY(cudaStreamSynchronize(s));
        if (ctx->pinned_u32[0] > copies) {
            first = level;
            break;
        }
    }
    CAC_CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
    CAC_CUDA_TRY(cudaStreamSynchronize(s));
    CAC_CUDA_TRY(cudaEventElapsedTime(&res->device_ms, ctx->ev[0], ctx->ev[1]));
    res->level = first;
    res->cut = 1ull << first;
    res->trials = copies * first;
    return CAC_OK;
}

}  // namespace cac
