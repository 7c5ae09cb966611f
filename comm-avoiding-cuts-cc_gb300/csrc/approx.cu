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
//
// The level count is the reference's ceil(ln w) of each rank's own slice weight (`w` at :19-30
// is the calling rank's local sum), the smallest over ranks: the ranks step through the levels'
// collectives together, so the reference's run is defined only while every rank is still in its
// loop, and the smallest count gives its answer wherever it has one.
//
// Seed replay (approx_run with ref_stream): the keep test instead consumes the reference's own
// draws. Rank r's engine is sitmo::prng_engine(seed + r) (ApproximateCut.hpp:35, .cpp:33), read in
// the reference's order: per level, for each copy, for each slice edge one
// std::binomial_distribution<int>(w, 2^-i) draw, then one raw output for the level's CC seed
// (:50-58). With w = 1 that draw (libstdc++'s waiting-time method) takes exactly one
// generate_canonical<double, 53> value U from the two outputs x0, x1 as (x0 + x1 2^32) / 2^64,
// and returns 1 iff -ln(1 - U) <= -ln(1 - 2^-i). So the draw for copy j and slice edge e of
// level i reads outputs k and k + 1, k = (i - 1) (2 C len_r + 1) + 2 (j len_r + e), and every
// edge of every copy is tested independently on the device. The test is an integer comparison
// of U 2^64 with a threshold per level (see stream_keep) that decides exactly as the logarithms
// do; no floating point runs on the device.
// Graphs with other weights draw a variable number of outputs per edge (a sequential chain per
// rank), so the replay takes unit weights only.
#include "cac_internal.h"
#include "sitmo.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

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

// Binomial(1, p) > 0 on the reference's draws: U = generate_canonical<double, 53> of outputs x0, x1
// (x0 + x1 2^32 rounded to a double, scaled by 2^-64, clamped below 1); kept iff
// -ln(1 - U) <= -ln(1 - p) (libstdc++'s waiting-time test with t = 1). ln is increasing, and for
// p = 2^-i <= 1/2 every double next to b = 1 - p lies at least two units in the last place of
// ln(b) away from it in logarithm, so any logarithm accurate to within one unit decides as
// fl(1 - U) >= b does. That test is made here in integers: with R = U 2^64 (x0 + x1 2^32 rounded
// to 53 significant bits, to nearest, ties to even), fl(1 - U) >= b iff 1 - R 2^-64 is at least
// the midpoint between b and the double below it (a tie rounds to b, whose significand is even
// for i <= 52), i.e. iff R <= T(i) with T(1) = 2^63 + 2^9 and T(i) = 2^(64-i) + 2^10 for
// 2 <= i <= 52 (levels stop at ceil(ln W) <= 45). R = 2^64 is U = 1, clamped below 1: never kept.
uint64_t stream_threshold(uint32_t level) {
    return level == 1 ? (1ull << 63) + (1ull << 9) : (1ull << (64 - level)) + (1ull << 10);
}

__device__ __forceinline__ bool stream_keep(uint64_t S, uint64_t T) {  // S = x0 + x1 2^32
    const int sh = 11 - __clzll(S);  // bits below the 53-bit significand
    if (sh <= 0) return S <= T;
    const uint64_t q = S >> sh, rem = S & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    const uint64_t qr = q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
    if (qr >> (64 - sh)) return false;
    return (qr << sh) <= T;
}

// Seed replay, unit weights: one thread per (copy, quad of 4 slice edges), quads numbered as in
// approx_keep_hook4. The quad's 4 draws read the 8 consecutive outputs k0 .. k0 + 7 of the rank's
// engine (output k = half k & 1 of word k >> 1, low half first: lib/prng_engine.hpp:195-212;
// words 4b .. 4b + 3 form sitmo block b). Draw d's two outputs give S = x0 + x1 2^32, which is
// word (k0 >> 1) + d itself when k0 is even and the high half of that word joined to the low half
// of the next when k0 is odd; the words lie in the blocks k0 >> 3 and the one after it.
__global__ void approx_stream_keep_hook(uint32_t *par, const uint32_t *__restrict__ U, const uint32_t *__restrict__ V,
                                        uint64_t m, uint32_t n, uint32_t level, uint64_t keep_max, uint32_t copies,
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
        const uint64_t base = (uint64_t)r * portion;
        const uint64_t len = r + 1 < ranks ? portion : m - base;
        const uint64_t k0 = (uint64_t)(level - 1) * (2 * (uint64_t)copies * len + 1) + 2 * ((uint64_t)j * len + 4 * lq);
        const uint64_t b0 = k0 >> 3;
        const unsigned a = (unsigned)(k0 >> 1) & 3u;  // first word inside block b0
        const bool odd = k0 & 1;
        const uint32_t key = seed + r;
        const u64x4 A = sitmo_block(key, 0, 0, 0, b0, 0, 0, 0);
        u64x4 B = A;
        if (a != 0 || odd) B = sitmo_block(key, 0, 0, 0, b0 + 1, 0, 0, 0);
        const uint64_t w[8] = {A.x[0], A.x[1], A.x[2], A.x[3], B.x[0], B.x[1], B.x[2], B.x[3]};
        uint64_t S[4];
#define CAC_QUAD_DRAWS(A0)                                                                     \
    _Pragma("unroll") for (int d = 0; d < 4; d++) S[d] =                                       \
        odd ? ((w[(A0) + d] >> 32) | (w[(A0) + d + 1] << 32)) : w[(A0) + d];
        switch (a) {
            case 0: CAC_QUAD_DRAWS(0) break;
            case 1: CAC_QUAD_DRAWS(1) break;
            case 2: CAC_QUAD_DRAWS(2) break;
            default: CAC_QUAD_DRAWS(3) break;
        }
#undef CAC_QUAD_DRAWS
#pragma unroll
        for (int d = 0; d < 4; d++) {
            const uint64_t local = 4 * lq + d;
            if (local >= len) break;
            if (!stream_keep(S[d], keep_max)) continue;
            aunite(par, U[base + local] + off, V[base + local] + off);
        }
    }
}

// Weight sum of every rank's slice. Slices as GraphInputIterator::loadSlice
// (src/input/GraphInputIterator.hpp:77-93): rank r < P - 1 owns [r portion, (r + 1) portion), the
// last rank the rest. Ranks along blockIdx.y (strided).
__global__ void approx_slice_sums(const uint32_t *__restrict__ w, uint64_t m, uint32_t ranks, uint64_t portion,
                                  unsigned long long *sums) {
    for (uint32_t r = blockIdx.y; r < ranks; r += gridDim.y) {
        const uint64_t from = (uint64_t)r * portion, to = r + 1 < ranks ? from + portion : m;
        unsigned long long acc = 0;
        for (uint64_t e = from + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < to;
             e += (uint64_t)gridDim.x * blockDim.x)
            acc += w[e];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if ((threadIdx.x & 31) == 0 && acc) atomicAdd(&sums[r], acc);
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

// ApproximateCut.cpp:30: (unsigned) ceil(log(w)), w a rank's slice weight (none for w = 0)
static uint32_t level_count(uint64_t w) { return w ? (uint32_t)std::ceil(std::log((double)w)) : 0; }

int approx_run(cac_ctx *ctx, const cac_graph *g, double p, uint32_t seed, uint32_t ranks, bool ref_stream,
               cac_approx_result *res) {
    cudaStream_t s = ctx->stream;
    *res = cac_approx_result{};
    const uint32_t copies = approx_copies(p);
    res->copies = copies;
    const uint64_t nv = (uint64_t)g->n * copies;
    if (nv >= 0xFFFFFFFFull) {
        set_error("approx_cut: n * copies must stay below 2^32");
        return CAC_ERR_UNSUPPORTED;
    }
    const uint64_t portion = g->m / ranks;
    if (ref_stream && !g->unit_weights) {
        set_error("approx_cut seed replay: every edge weight must be 1 (a weighted edge draws a variable number "
                  "of outputs)");
        return CAC_ERR_UNSUPPORTED;
    }
    // Levels: the smallest ceil(ln w_r) over the ranks' slices. More ranks than edges leave every
    // slice but the last empty: no level runs. Unit weights: w_r is the slice length; one rank:
    // the graph's total weight; otherwise the slice sums are taken on the device.
    const bool stats = ranks > 1 && portion > 0 && !g->unit_weights;
    CAC_TRY(arena_reserve(ctx, align_up(nv * 4 + 4) + 256 + (stats ? align_up((uint64_t)ranks * 8) : 0)));
    arena_reset(ctx);
    uint32_t *par = (uint32_t *)arena_take(ctx, nv * 4 + 4);
    unsigned int *d_count = (unsigned int *)arena_take(ctx, 16);
    CAC_CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
    uint32_t iterations = level_count(g->total_weight);
    if (ranks > 1 && portion == 0) {
        iterations = 0;
    } else if (ranks > 1 && g->unit_weights) {
        iterations = level_count(portion);  // the last slice holds at least `portion` edges
    } else if (stats) {
        unsigned long long *d_sums = (unsigned long long *)arena_take(ctx, (uint64_t)ranks * 8);
        CAC_CUDA_TRY(cudaMemsetAsync(d_sums, 0, (uint64_t)ranks * 8, s));
        const uint64_t longest = g->m - (uint64_t)(ranks - 1) * portion;
        const uint32_t gy = std::min<uint32_t>(ranks, 65535u);
        const uint32_t gx = (uint32_t)std::max<uint64_t>(
            1, std::min<uint64_t>((longest + 4 * kThreads - 1) / (4 * kThreads),
                                  std::max<uint64_t>(1, (uint64_t)ctx->num_sms * 8 / gy)));
        approx_slice_sums<<<dim3(gx, gy), kThreads, 0, s>>>(g->w, g->m, ranks, portion, d_sums);
        CAC_CUDA_TRY(cudaGetLastError());
        std::vector<unsigned long long> h(ranks);  // ranks <= m here
        CAC_CUDA_TRY(cudaMemcpyAsync(h.data(), d_sums, (uint64_t)ranks * 8, cudaMemcpyDeviceToHost, s));
        CAC_CUDA_TRY(cudaStreamSynchronize(s));
        iterations = UINT32_MAX;
        for (uint32_t r = 0; r < ranks; r++) iterations = std::min(iterations, level_count(h[r]));
    }
    // quads of 4 edges per rank slice (see approx_keep_hook4)
    const uint64_t Qf = (portion + 3) / 4;
    const uint64_t Q = portion == 0 ? (g->m + 3) / 4 : (ranks - 1) * Qf + (g->m - (uint64_t)(ranks - 1) * portion + 3) / 4;
    const int gi = (int)std::max<uint64_t>(1, std::min<uint64_t>((nv + kThreads - 1) / kThreads, ctx->num_sms * 8));
    uint32_t first = 0;
    if (ref_stream) iterations = std::min<uint32_t>(iterations, 52);  // ceil(ln W) <= 45 for W < 2^64
    for (uint32_t level = 1; level <= iterations && level <= 63; level++) {
        approx_init<<<gi, kThreads, 0, s>>>(par, nv);
        // the kept edges are hooked in kSlices slices, the forest flattened after the first few
        // and the last (the same partition as one pass; one pass from singletons builds long
        // parent chains on large graphs)
        if (ref_stream) {
            const uint64_t keep_max = stream_threshold(level);  // p = 2^-level (ApproximateCut.cpp:37)
            const uint32_t slices = Q < (1u << 16) ? 1 : kSlices;
            for (uint32_t sl = 0; sl < slices; sl++) {
                const uint64_t q0 = Q * sl / slices, q1 = Q * (sl + 1) / slices;
                if (q1 <= q0) continue;
                const int ge = (int)std::max<uint64_t>(
                    1, std::min<uint64_t>((q1 - q0 + kThreads - 1) / kThreads,
                                          std::max(1, ctx->num_sms * 8 / (int)copies)));
                approx_stream_keep_hook<<<dim3(ge, copies), kThreads, 0, s>>>(par, g->u, g->v, g->m, g->n, level,
                                                                              keep_max, copies, seed, ranks,
                                                                              portion, Qf, q0, q1);
                if (sl < kCompressedSlices && sl + 1 < slices) approx_compress<<<gi, kThreads, 0, s>>>(par, nv);
            }
        } else if (Q < (1u << 16)) {
            if (g->m) {
                const int ge = (int)std::max<uint64_t>(
                    1, std::min<uint64_t>((g->m + kThreads - 1) / kThreads, std::max(1, ctx->num_sms * 8 / (int)copies)));
                dim3 grid(ge, copies);
                approx_keep_hook<<<grid, kThreads, 0, s>>>(par, g->u, g->v, g->w, g->m, g->n, level, seed, ranks,
                                                           portion);
            }
        }
        const uint32_t slices = ref_stream || Q < (1u << 16) ? 0 : kSlices;
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
