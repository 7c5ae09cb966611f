// Connected components: the GB300 form of the reference's iterated-sparse-sampling CC
// (src/UnweightedIteratedSparseSampling.cpp:40-72, src/IteratedSparseSampling.hpp:160-295).
//
// Reference round structure            ->  here
//   root scatters per-rank draw counts    host restates edgesToSamplePerProcessor (cc_plan)
//   rank r draws engine()%slice samples   cc_sample_hook: sitmo stream (seed + r, 0, 0, 0),
//     with sitmo(seed + r)                  output k = word k % 8 of block k / 8, exactly the
//                                           reference's k-th draw; every draw hooks its edge
//   root: shuffle + prefix union-find     lock-free union-find in HBM (atomicCAS hooking of
//     to one component (Boost sets)         the larger root under the smaller, so roots are
//                                           component minima; order-free for target 1)
//   bcast map, rewrite slice, drop loops  cc_edge_pass: one streaming pass over every edge;
//     and repeat while edges remain         edges whose endpoints already share a root are the
//                                           dropped loops, the rest hook (the final round)
//   relabel by first appearance           roots = minima, so label = exclusive scan of the
//                                           root flags (cc_finalize_count/scan/rank/label)
//
// Memory layout in HBM: edge endpoints as two uint32 arrays u[m], v[m] (structure of arrays,
// 16-byte vector loads, 4 edges per load pair); parent[n] uint32 (L2-resident for n up to
// tens of millions: 129 MB of L2); per-tile root counts; labels[n].
#include "cac_internal.h"
#include "sitmo.cuh"

#include <algorithm>
#include <cmath>

namespace cac {
namespace {

constexpr int kThreads = 256;
constexpr int kTileItems = 16;                       // vertices per thread in the labelling tiles
constexpr int kTile = kThreads * kTileItems;         // vertices per labelling tile
constexpr size_t kPinnedBytes = 60 * 1024;           // ctx pinned staging available for rank descriptors
constexpr int kEdgeThreads = 1024;                   // closing-pass CTA (one per SM: the bitmap fills smem)
constexpr uint32_t kSmemBitmapWords = 48 * 1024;     // 192 KB of bitmap in shared memory (1.57M vertices)
constexpr uint32_t kGiantSample = 4096;              // vertices sampled to find the giant component

struct RankDesc {
    uint64_t slice_off;
    uint64_t slice_len;
    uint64_t draws;
    uint64_t block_off;  // first sitmo block of this rank in the flattened launch
    uint32_t key0;       // seed + rank
    uint32_t pad;
};

// Root of v with path halving. Invariant: parent[x] <= x, roots satisfy parent[r] == r.
__device__ __forceinline__ uint32_t find_root(uint32_t *par, uint32_t v) {
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

// Root of v without writes. Used where no hooking happens any more: a path-halving write by
// one thread could otherwise overwrite another thread's just-stored `parent[i] = root` with a
// non-root ancestor and leave i uncompressed.
__device__ __forceinline__ uint32_t find_root_ro(const uint32_t *par, uint32_t v) {
    uint32_t cur = v, next;
    while ((next = par[cur]) != cur) cur = next;
    return cur;
}

// Merge the sets of a and b: hook the larger representative under the smaller with CAS;
// a failed CAS returns the node's new parent and the walk continues from there.
__device__ __forceinline__ void unite(uint32_t *par, uint32_t a, uint32_t b) {
    uint32_t ra = find_root(par, a), rb = find_root(par, b);
    while (ra != rb) {
        if (ra < rb) {
            uint32_t old = atomicCAS(&par[rb], rb, ra);
            if (old == rb) return;
            rb = old;
        } else {
            uint32_t old = atomicCAS(&par[ra], ra, rb);
            if (old == ra) return;
            ra = old;
        }
    }
}

__global__ void cc_init(uint32_t *par, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) par[i] = i;
}

// One thread per sitmo block (8 draws of one virtual rank).
__global__ void cc_sample_hook(uint32_t *par, const uint32_t *__restrict__ u, const uint32_t *__restrict__ v,
                               const RankDesc *__restrict__ ranks, int nranks, uint64_t total_blocks) {
    for (uint64_t blk = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; blk < total_blocks;
         blk += (uint64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = nranks - 1;  // last rank whose block_off <= blk
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (ranks[mid].block_off <= blk) lo = mid; else hi = mid - 1;
        }
        const RankDesc rd = ranks[lo];
        const uint64_t local = blk - rd.block_off;
        const u64x4 o = sitmo_block(rd.key0, 0, 0, 0, local, 0, 0, 0);
        const uint64_t first = local * 8;
        const uint32_t len = (uint32_t)rd.slice_len;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            if (first + j >= rd.draws) break;
            const uint64_t word = o.x[j >> 1];
            const uint32_t x = (j & 1) ? (uint32_t)(word >> 32) : (uint32_t)word;
            const uint64_t e = rd.slice_off + (rd.slice_len > 0xFFFFFFFFull ? (uint64_t)x : (uint64_t)(x % len));
            unite(par, __ldg(u + e), __ldg(v + e));
        }
    }
}

__global__ void cc_compress(uint32_t *par, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        par[i] = find_root_ro(par, i);
}

__device__ __forceinline__ void edge_hook(uint32_t *par, uint32_t a, uint32_t b) {
    const uint32_t pa = par[a], pb = par[b];
    if (pa == pb) return;  // already one component: the reference drops this edge as a loop
    unite(par, pa, pb);
}

// The most frequent root among kGiantSample vertices spread over [0, n) (compressed parents):
// one CTA sorts the sampled roots in shared memory and takes the longest run.
__global__ void __launch_bounds__(1024) cc_find_giant(const uint32_t *par, uint32_t n, uint32_t *giant) {
    __shared__ uint32_t r[kGiantSample];
    for (uint32_t i = threadIdx.x; i < kGiantSample; i += blockDim.x) {
        const uint64_t v = ((uint64_t)i * 2654435761u) % n;  // fixed spread of sample positions
        r[i] = par[v];
    }
    __syncthreads();
    // bitonic sort of kGiantSample (power of two) keys
    for (uint32_t k = 2; k <= kGiantSample; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < kGiantSample; i += blockDim.x) {
                const uint32_t p = i ^ j;
                if (p > i) {
                    const bool up = (i & k) == 0;
                    const uint32_t a = r[i], b = r[p];
                    if ((a > b) == up) { r[i] = b; r[p] = a; }
                }
            }
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) {
        uint32_t best = r[0], best_len = 0, run = 0;
        for (uint32_t i = 0; i < kGiantSample; i++) {
            run = (i > 0 && r[i] == r[i - 1]) ? run + 1 : 1;
            if (run > best_len) { best_len = run; best = r[i]; }
        }
        *giant = best;
    }
}

// bit v of the bitmap = (parent[v] == giant root), one warp ballot per 32 vertices
__global__ void cc_giant_bitmap(const uint32_t *par, uint32_t n, const uint32_t *giant, uint32_t *bits) {
    const uint32_t g = *giant;
    const uint64_t nw = ((uint64_t)n + 31) / 32;
    const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nw; w += warps) {
        const uint64_t v = w * 32 + (threadIdx.x & 31);
        const bool in = v < n && par[v] == g;
        const uint32_t word = __ballot_sync(0xffffffffu, in);
        if ((threadIdx.x & 31) == 0) bits[w] = word;
    }
}

__device__ __forceinline__ bool in_giant(const uint32_t *sbits, uint32_t swords, const uint32_t *gbits, uint32_t x) {
    const uint32_t w = x >> 5;
    const uint32_t word = w < swords ? sbits[w] : __ldg(gbits + w);
    return (word >> (x & 31)) & 1u;
}

template <bool kSkip>
__device__ __forceinline__ void visit_edge(uint32_t *par, const uint32_t *sbits, uint32_t swords,
                                           const uint32_t *gbits, uint32_t a, uint32_t b) {
    if (kSkip && in_giant(sbits, swords, gbits, a) && in_giant(sbits, swords, gbits, b)) return;  // same component
    edge_hook(par, a, b);
}

// Closing pass over every edge, 4 edges per thread step through 16-byte streaming loads. The
// membership bitmap of the giant component (its first `swords` words staged in shared memory,
// the rest read through the read-only path) lets edges inside the giant component skip the
// parent lookups entirely.
template <bool kVec, bool kSkip>
__global__ void __launch_bounds__(kEdgeThreads) cc_edge_pass(uint32_t *par, const uint32_t *__restrict__ u,
                                                             const uint32_t *__restrict__ v, uint64_t m,
                                                             const uint32_t *__restrict__ gbits, uint32_t nwords) {
    extern __shared__ uint32_t sbits[];
    const uint32_t swords = kSkip ? min(nwords, (uint32_t)kSmemBitmapWords) : 0;
    for (uint32_t i = threadIdx.x; i < swords; i += blockDim.x) sbits[i] = gbits[i];
    __syncthreads();
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t done = 0;
    if (kVec) {
        const uint64_t m4 = m >> 2;
        const uint4 *u4 = reinterpret_cast<const uint4 *>(u);
        const uint4 *v4 = reinterpret_cast<const uint4 *>(v);
        for (uint64_t i = tid; i < m4; i += stride) {
            const uint4 a = __ldcs(u4 + i);
            const uint4 b = __ldcs(v4 + i);
            visit_edge<kSkip>(par, sbits, swords, gbits, a.x, b.x);
            visit_edge<kSkip>(par, sbits, swords, gbits, a.y, b.y);
            visit_edge<kSkip>(par, sbits, swords, gbits, a.z, b.z);
            visit_edge<kSkip>(par, sbits, swords, gbits, a.w, b.w);
        }
        done = m4 << 2;
    }
    for (uint64_t e = done + tid; e < m; e += stride)
        visit_edge<kSkip>(par, sbits, swords, gbits, __ldcs(u + e), __ldcs(v + e));
}

__device__ __forceinline__ uint32_t block_sum(uint32_t x, uint32_t *sh) {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = x;
    __syncthreads();
    uint32_t t = 0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    return t;  // valid in thread 0
}

// Final compression, root flags and per-tile root counts.
__global__ void __launch_bounds__(kThreads) cc_finalize_count(uint32_t *par, uint32_t n, uint32_t *tile_counts) {
    __shared__ uint32_t sh[32];
    const uint64_t base = (uint64_t)blockIdx.x * kTile;
    uint32_t c = 0;
#pragma unroll 4
    for (int k = 0; k < kTileItems; k++) {
        const uint64_t i = base + (uint64_t)k * kThreads + threadIdx.x;
        if (i < n) {
            const uint32_t r = find_root_ro(par, (uint32_t)i);
            par[i] = r;
            c += (r == (uint32_t)i);
        }
    }
    const uint32_t t = block_sum(c, sh);
    if (threadIdx.x == 0) tile_counts[blockIdx.x] = t;
}

// Exclusive scan of the tile counts by one block, chunk by chunk; writes the total.
__global__ void __launch_bounds__(1024) cc_scan_tiles(const uint32_t *counts, uint32_t *offsets, uint32_t ntiles,
                                                      uint32_t *total) {
    __shared__ uint32_t sh[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < ntiles; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t x = i < ntiles ? counts[i] : 0;
        // inclusive warp scan
        uint32_t s = x;
        const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (l >= o) s += y;
        }
        if (l == 31) sh[w] = s;
        __syncthreads();
        if (w == 0) {
            uint32_t t = l < (int)(blockDim.x >> 5) ? sh[l] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
                if (l >= o) t += y;
            }
            sh[l] = t;
        }
        __syncthreads();
        const uint32_t warp_off = w ? sh[w - 1] : 0;
        if (i < ntiles) offsets[i] = carry + warp_off + s - x;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += warp_off + s;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

// Rank of every root: tile offset + exclusive scan of root flags inside the tile.
__global__ void __launch_bounds__(kThreads) cc_rank_roots(const uint32_t *par, uint32_t n, const uint32_t *offsets,
                                                          uint32_t *labels) {
    __shared__ uint32_t sh[32];
    const uint64_t base = (uint64_t)blockIdx.x * kTile + (uint64_t)threadIdx.x * kTileItems;
    uint32_t flags = 0, c = 0;
#pragma unroll
    for (int k = 0; k < kTileItems; k++) {
        const uint64_t i = base + k;
        const uint32_t f = (i < n) && par[i] == (uint32_t)i;
        flags |= f << k;
        c += f;
    }
    // exclusive scan of c over the block (thread order == vertex order inside the tile)
    uint32_t s = c;
    const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
        if (l >= o) s += y;
    }
    if (l == 31) sh[w] = s;
    __syncthreads();
    if (w == 0) {
        uint32_t t = l < (kThreads >> 5) ? sh[l] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (l >= o) t += y;
        }
        sh[l] = t;
    }
    __syncthreads();
    uint32_t r = offsets[blockIdx.x] + (w ? sh[w - 1] : 0) + s - c;
#pragma unroll
    for (int k = 0; k < kTileItems; k++) {
        if ((flags >> k) & 1u) labels[base + k] = r++;
    }
}

__global__ void cc_label_all(const uint32_t *par, uint32_t n, uint32_t *labels) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t r = par[i];
        if (r != i) labels[i] = labels[r];
    }
}

int grid_for(cac_ctx *ctx, uint64_t work, int per_sm) {
    const uint64_t need = (work + kThreads - 1) / kThreads;
    const uint64_t cap = (uint64_t)ctx->num_sms * per_sm;
    return (int)std::max<uint64_t>(1, std::min(need, cap));
}

}  // namespace

CCPlan cc_plan(uint32_t n, uint64_t m, uint32_t ranks) {
    // UnweightedIteratedSparseSampling::loadSlice (.cpp:5-21) and edgesToSamplePerProcessor
    // (.cpp:80-128), same float expressions and uint32 wrap-around.
    CCPlan p;
    p.slice_off.resize(ranks);
    p.slice_len.resize(ranks);
    p.draws.assign(ranks, 0);
    const uint64_t portion = m / ranks;
    std::vector<int> avail(ranks), per(ranks, 0);
    uint32_t total = 0;
    for (uint32_t r = 0; r < ranks; r++) {
        p.slice_off[r] = portion * r;
        p.slice_len[r] = (r == ranks - 1) ? m - portion * r : portion;
        avail[r] = (int)p.slice_len[r];
        total += (uint32_t)avail[r];
    }
    const uint32_t want = (uint32_t)(std::pow((float)n, 1.0f + 0.09f / 2) * (1.0f + 0.2f));
    uint32_t to_sample = std::min(want, total);
    const uint32_t threshold = (uint32_t)(3.0f / (0.2f * 0.2f) * std::log((float)ranks / 0.9f));
    uint32_t remaining = to_sample;
    for (uint32_t i = 0; i < ranks; i++) {
        if ((uint32_t)avail[i] <= threshold) {
            per[i] = avail[i];
            remaining -= (uint32_t)avail[i];
            to_sample -= (uint32_t)avail[i];
        }
    }
    for (uint32_t i = 0; i < ranks; i++) {
        if (per[i] != 0) continue;
        const int share = (int)((float)to_sample * (float)avail[i] / (float)total);
        per[i] = std::min(share, avail[i]);
        remaining -= (uint32_t)per[i];
    }
    for (uint32_t sp = 0; remaining > 0 && sp < ranks; sp++) {
        if (avail[sp] > per[sp]) {
            const uint32_t delta = std::min((uint32_t)(avail[sp] - per[sp]), remaining);
            per[sp] += (int)delta;
            remaining -= delta;
        }
    }
    for (uint32_t r = 0; r < ranks; r++) {
        // a rank asked for its whole slice returns the slice itself (.cpp:28-29): those edges
        // are covered by the closing pass, so nothing is drawn for it.
        p.draws[r] = ((uint64_t)per[r] == p.slice_len[r]) ? 0 : (uint64_t)per[r];
    }
    return p;
}

size_t cc_scratch_bytes(uint32_t n, uint32_t ranks) {
    const size_t ntiles = ((size_t)n + kTile - 1) / kTile;
    const size_t nwords = ((size_t)n + 31) / 32;
    return align_up((size_t)n * 4) + 2 * align_up(ntiles * 4 + 4) + align_up(256) +
           align_up(sizeof(RankDesc) * (size_t)ranks) + align_up(nwords * 4 + 4);
}

int cc_run(cac_ctx *ctx, uint32_t n, uint64_t m, const uint32_t *d_u, const uint32_t *d_v, uint32_t seed,
           uint32_t ranks, uint32_t *d_labels, cac_cc_result *res) {
    if (ranks == 0) ranks = 1;
    cudaStream_t s = ctx->stream;
    CAC_CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
    if (n == 0) {
        if (res) { *res = cac_cc_result{}; }
        return CAC_OK;
    }
    const CCPlan plan = cc_plan(n, m, ranks);
    const uint32_t ntiles = (uint32_t)(((uint64_t)n + kTile - 1) / kTile);

    CAC_TRY(arena_reserve(ctx, cc_scratch_bytes(n, ranks)));
    arena_reset(ctx);
    uint32_t *par = (uint32_t *)arena_take(ctx, (size_t)n * 4);
    uint32_t *counts = (uint32_t *)arena_take(ctx, (size_t)ntiles * 4 + 4);
    uint32_t *offsets = (uint32_t *)arena_take(ctx, (size_t)ntiles * 4 + 4);
    uint32_t *total = (uint32_t *)arena_take(ctx, 256);
    uint32_t *giant = total + 8;
    RankDesc *d_ranks = (RankDesc *)arena_take(ctx, sizeof(RankDesc) * ranks);
    const uint32_t nwords = (uint32_t)(((uint64_t)n + 31) / 32);
    uint32_t *bits = (uint32_t *)arena_take(ctx, (size_t)nwords * 4 + 4);

    // rank descriptors go through the ctx's pinned staging page when they fit (async copy)
    std::vector<RankDesc> hv;
    RankDesc *hr = nullptr;
    const bool pinned = sizeof(RankDesc) * ranks <= kPinnedBytes;
    if (pinned) {
        hr = reinterpret_cast<RankDesc *>(ctx->pinned_u32 + 64);
    } else {
        hv.resize(ranks);
        hr = hv.data();
    }
    uint64_t blocks = 0, drawn = 0;
    for (uint32_t r = 0; r < ranks; r++) {
        hr[r].slice_off = plan.slice_off[r];
        hr[r].slice_len = plan.slice_len[r];
        hr[r].draws = plan.draws[r];
        hr[r].block_off = blocks;
        hr[r].key0 = seed + r;
        hr[r].pad = 0;
        blocks += (plan.draws[r] + 7) / 8;
        drawn += plan.draws[r];
    }

    cc_init<<<grid_for(ctx, n, 8), kThreads, 0, s>>>(par, n);
    if (blocks > 0 && m > 0) {
        CAC_CUDA_TRY(cudaMemcpyAsync(d_ranks, hr, sizeof(RankDesc) * ranks, cudaMemcpyHostToDevice, s));
        cc_sample_hook<<<grid_for(ctx, blocks, 8), kThreads, 0, s>>>(par, d_u, d_v, d_ranks, (int)ranks, blocks);
        cc_compress<<<grid_for(ctx, n, 8), kThreads, 0, s>>>(par, n);
        cc_find_giant<<<1, 1024, 0, s>>>(par, n, giant);
        cc_giant_bitmap<<<grid_for(ctx, n, 8), kThreads, 0, s>>>(par, n, giant, bits);
    }
    CAC_CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
    if (m > 0) {
        const bool vec = ((reinterpret_cast<uintptr_t>(d_u) | reinterpret_cast<uintptr_t>(d_v)) & 15) == 0;
        const bool skip = blocks > 0;  // a sampling round ran, so a giant component exists
        const size_t sm = skip ? (size_t)std::min(nwords, kSmemBitmapWords) * 4 : 0;
        const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)ctx->num_sms * (skip ? 1 : 2),
                                                                        (m + 4 * kEdgeThreads - 1) / (4 * kEdgeThreads)));
        auto launch = [&](auto kernel) -> int {
            CAC_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
            kernel<<<grid, kEdgeThreads, sm, s>>>(par, d_u, d_v, m, bits, nwords);
            return CAC_OK;
        };
        if (vec && skip) CAC_TRY(launch(cc_edge_pass<true, true>));
        else if (vec) CAC_TRY(launch(cc_edge_pass<true, false>));
        else if (skip) CAC_TRY(launch(cc_edge_pass<false, true>));
        else CAC_TRY(launch(cc_edge_pass<false, false>));
    }
    CAC_CUDA_TRY(cudaEventRecord(ctx->ev[2], s));
    cc_finalize_count<<<ntiles, kThreads, 0, s>>>(par, n, counts);
    cc_scan_tiles<<<1, 1024, 0, s>>>(counts, offsets, ntiles, total);
    if (d_labels) {
        cc_rank_roots<<<ntiles, kThreads, 0, s>>>(par, n, offsets, d_labels);
        cc_label_all<<<grid_for(ctx, n, 8), kThreads, 0, s>>>(par, n, d_labels);
    }
    CAC_CUDA_TRY(cudaGetLastError());
    CAC_CUDA_TRY(cudaMemcpyAsync(ctx->pinned_u32, total, 4, cudaMemcpyDeviceToHost, s));
    CAC_CUDA_TRY(cudaEventRecord(ctx->ev[3], s));
    CAC_CUDA_TRY(cudaStreamSynchronize(s));
    if (res) {
        res->num_components = ctx->pinned_u32[0];
        res->rounds = (blocks > 0 ? 1u : 0u) + (m > 0 ? 1u : 0u);
        res->sampled_edges = drawn;
        CAC_CUDA_TRY(cudaEventElapsedTime(&res->device_ms, ctx->ev[0], ctx->ev[3]));
        CAC_CUDA_TRY(cudaEventElapsedTime(&res->edge_pass_ms, ctx->ev[1], ctx->ev[2]));
    }
    return CAC_OK;
}

}  // namespace cac
