// approx_cut: the GB300 form of ApproximateCut::run (src/ApproximateCut.cpp:10-79).
//
// For levels i = 1 .. ceil(ln W) the reference keeps each edge of each of `copies` disjoint
// copies iff Binomial(w, 2^-i) > 0 (std::binomial_distribution, :39-48), relabels copy j to
// v + j n, runs the iterated-sparse-sampling CC on the union and stops at the first level with
// more than `copies` components; the answer is 2^level.
//
// Here each level does the keep test of every (copy, edge) pair and hooks kept edges straight
// into one union-find over n * copies vertices, in slices with the forest flattened between the
// first ones (the CC of the disjoint union is the
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
constexpr uint32_t kSlices = 8;            // hook slices per level on large graphs
constexpr uint32_t kCompressedSlices = 3;  // slices followed by a full compression

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

// One thread per (copy, edge), one sitmo block per draw: small graphs, where the pass is one
// latency chain per thread and more threads finish sooner. Copies along blockIdx.y.
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

// Large graphs: one thread per (copy, quad): a quad is 4 consecutive edges of one rank's slice, local indices
// 4 lq .. 4 lq + 3, whose 4 draws are the 4 words of one sitmo block (counter lq). Rank r < P - 1
// owns Qf = ceil(portion / 4) quads, the last rank the rest of the edges (all of them when
// portion is 0). Quads [q0, q1) of the flattened list; copies along blockIdx.y.
__global__ void approx_keep_hook4(uint32_t *par, const uint32_t *__restrict__ U, const uint32_t *__restrict__ V,
                                  const uint32_t *__restrict__ Wt, uint64_t m, uint32_t n, uint32_t level,
                                  uint32_t seed, uint32_t ranks, uint64_t portion, uint64_t Qf, uint64_t q0,
                                  uint64_t q1) {
    const uint32_t j = blockIdx.y;
    const uint32_t off = j * n;
    for (uint64_t gq = q0 + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; gq < q1;
         gq += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t r;
        uint64_t lq;
        if (portion == 0) {
            r = ranks - 1;
            lq = gq;
        } else {
            const uint64_t rr = gq / Qf;
            r = rr < ranks - 1 ? (uint32_t)rr : ranks - 1;
            lq = gq - (uint64_t)r * Qf;
        }
        const uint64_t base = (uint64_t)r * portion;                   // first edge of the slice
        const uint64_t len = r + 1 < ranks ? portion : m - base;       // edges of the slice
        const u64x4 o = sitmo_block(seed + r, level, j, 1, lq, 0, 0, 0);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const uint64_t local = 4 * lq + k;
            if (local >= len) break;
            const uint64_t e = base + local;
            const uint32_t w = Wt[e];
            if (w == 0 || o.x[k] < keep_threshold(level, w)) continue;
            aunite(par, U[e] + off, V[e] + off);
        }
    }
}

// Full path compression (read-only walks; only roots are written).
__global__ void approx_compress(uint32_t *par, uint64_t nv) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t cur = par[i], next;
        if (cur == (uint32_t)i) continue;
        while ((next = par[cur]) != cur) cur = next;
        par[i] = cur;
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
    // quads of 4 edges per rank slice (see approx_keep_hook4)
    const uint64_t Qf = (portion + 3) / 4;
    const uint64_t Q = portion == 0 ? (g->m + 3) / 4 : (ranks - 1) * Qf + (g->m - (uint64_t)(ranks - 1) * portion + 3) / 4;
    const int gi = (int)std::max<uint64_t>(1, std::min<uint64_t>((nv + kThreads - 1) / kThreads, ctx->num_sms * 8));
    CAC_CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
    uint32_t first = 0;
    for (uint32_t level = 1; level <= iterations && level <= 63; level++) {
        approx_init<<<gi, kThreads, 0, s>>>(par, nv);
        // the kept edges are hooked in kSlices slices, the forest flattened after the first few
        // and the last (the same partition as one pass; one pass from singletons builds long
        // parent chains on large graphs)
        if (Q < (1u << 16)) {
            if (g->m) {
                const int ge = (int)std::max<uint64_t>(
                    1, std::min<uint64_t>((g->m + kThreads - 1) / kThreads, std::max(1, ctx->num_sms * 8 / (int)copies)));
                dim3 grid(ge, copies);
                approx_keep_hook<<<grid, kThreads, 0, s>>>(par, g->u, g->v, g->w, g->m, g->n, level, seed, ranks,
                                                           portion);
            }
        }
        const uint32_t slices = Q < (1u << 16) ? 0 : kSlices;
        for (uint32_t sl = 0; sl < slices; sl++) {
            const uint64_t q0 = Q * sl / slices, q1 = Q * (sl + 1) / slices;
            if (q1 <= q0) continue;
            const int ge = (int)std::max<uint64_t>(
                1, std::min<uint64_t>((q1 - q0 + kThreads - 1) / kThreads, std::max(1, ctx->num_sms * 8 / (int)copies)));
            dim3 grid(ge, copies);
            approx_keep_hook4<<<grid, kThreads, 0, s>>>(par, g->u, g->v, g->w, g->m, g->n, level, seed, ranks, portion,
                                                        Qf, q0, q1);
            if (sl < kCompressedSlices && sl + 1 < slices) approx_compress<<<gi, kThreads, 0, s>>>(par, nv);
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
