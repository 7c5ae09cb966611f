// Connected components: the GB300 form of the reference's iterated-sparse-sampling CC
// (src/UnweightedIteratedSparseSampling.cpp:40-72, src/IteratedSparseSampling.hpp:160-295).
//
// Reference round structure            ->  here
//   root scatters per-rank draw counts    host restates edgesToSamplePerProcessor (cc_plan)
//   rank r draws engine()%slice samples   cc_sample_draws / cc_sample_hook: sitmo stream
//     with sitmo(seed + r)                  (seed + r, 0, 0, 0), output k = word k % 8 of block
//                                           k / 8, the reference's k-th engine output; it picks
//                                           a 32-edge chunk of the slice (coalesced) instead of
//                                           one edge
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
#include <mutex>
#include <string>

namespace cac {
namespace {

// Programmatic dependent launch: a kernel launched with launch_pdl may start while its predecessor
// on the stream drains; pdl_wait() (griddepcontrol.wait) holds it until the predecessor has
// completed and its writes are visible, so every kernel calls it before its first dependent
// access. After an ordinary launch it returns at once. Measured on the CC query (22 kernels in
// one replayed graph): BA n=1,024,000 194.9 -> 192.8 us, R-MAT scale 22 about 1-3 us.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

constexpr int kThreads = 256;
constexpr int kTileItems = 4;                        // vertices per thread in the labelling tiles
constexpr int kTile = kThreads * kTileItems;         // vertices per labelling tile
constexpr size_t kPinnedBytes = 60 * 1024;           // ctx pinned staging available for rank descriptors
constexpr int kEdgeThreads = 1024;                   // closing-pass CTA (one per SM: the bitmap fills smem)
constexpr uint32_t kSmemBitmapWords = 48 * 1024;     // 192 KB of bitmap in shared memory (1.57M vertices)
constexpr uint32_t kGiantSample = 1024;              // vertices sampled to find the giant component
constexpr uint32_t kSampleChunk = 32;                // consecutive edges behind one sampling draw
// Slices of the sampling round, in eighths of its draws: a first slice above an eighth builds long
// parent chains from the singletons (2/8 first: 451 vs 209 us per BA n=1,024,000 query), later
// ones mostly hook small trees onto the giant one and can be larger. Every slice but the last is
// followed by a full compression; the last by the fused compression + giant search + bitmap.
// Measured per BA n=1,024,000 query against eight even slices (compressions after the first three
// and the last): 1,1,2,4 202.0 vs 208.8 us; 1,1,1,5 203.3; 1,1,1,1,4 206.6; 1,1,1,1,1,3 204.9.
// R-MAT scale 22: 1,1,1,5 647.5 vs 666.4 us.
constexpr uint32_t kSliceEighths[] = {1, 1, 2, 4};
constexpr uint32_t kMaxRegions = 1024;               // filter CTAs (regions of the survivor buffer)
// survivor-hook CTAs per SM: about one survivor per thread on BA n=1,024,000 (0.6 M survivors);
// 8 against 4: 20 vs 22.5 us there, 47 vs 63.5 us on R-MAT scale 22; 16 no better
constexpr unsigned kSurvivorBlocksPerSm = 8;
constexpr uint32_t kStreamPieces = 8;                // sample pieces (and gaps) of a host edge list
constexpr uint32_t kErrWord = 9;                     // a query's error word (after its count and giant root)
constexpr uint32_t kErrBadId = 1;                    // an edge endpoint was >= n (the edge was skipped)

struct RankDesc {
    uint64_t slice_off;
    uint64_t slice_len;
    uint64_t draws;      // chunk draws of this rank
    uint64_t block_off;  // first sitmo block (8 chunk draws) of this rank in the flattened launch
    uint64_t draw_off;   // first chunk draw of this rank in the flattened draw list
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

__device__ __forceinline__ void edge_hook(uint32_t *par, uint32_t a, uint32_t b) {
    const uint32_t pa = par[a], pb = par[b];
    if (pa == pb) return;  // already one component: the reference drops this edge as a loop
    unite(par, pa, pb);
}

// Edge lists handed in by the caller (host arrays of cac_cc_edges, device arrays of
// cac_cc_noalloc) are not validated beforehand: an endpoint >= n skips the edge and sets the
// query's error word instead of indexing past the parent array.
template <bool kCheck>
__device__ __forceinline__ void edge_hook_checked(uint32_t *par, uint32_t a, uint32_t b, uint32_t n, uint32_t *err) {
    if (kCheck && (a >= n || b >= n)) {
        atomicOr(err, kErrBadId);
        return;
    }
    edge_hook(par, a, b);
}

__global__ void cc_init(uint32_t *par, uint32_t n) {
    pdl_wait();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) par[i] = i;
}

// The draws of the sampling round, one thread per sitmo block (8 draws of one rank). The reference
// draws single edges (engine() % slice, a random 8-byte gather each); here draw k of rank r
// (32-bit output k of stream (seed + r, 0, 0, 0), word k % 8 of block k / 8) selects chunk
// (output % chunks) of kSampleChunk consecutive edges of the rank's slice. The chunk is stored as
// (first edge | edge count << 32) at the draw's flattened index.
__global__ void cc_sample_draws(const RankDesc *__restrict__ ranks, int nranks, uint64_t nblocks,
                                uint64_t *__restrict__ chunks) {
    pdl_wait();
    for (uint64_t gb = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; gb < nblocks;
         gb += (uint64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = nranks - 1;  // last rank whose first block <= gb
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (ranks[mid].block_off <= gb) lo = mid; else hi = mid - 1;
        }
        const RankDesc rd = ranks[lo];
        const uint64_t blk = gb - rd.block_off;  // sitmo block index within the rank's stream
        const u64x4 o = sitmo_block(rd.key0, 0, 0, 0, blk, 0, 0, 0);
        const uint64_t nchunks = (rd.slice_len + kSampleChunk - 1) / kSampleChunk;
        const uint64_t end = rd.slice_off + rd.slice_len;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const uint64_t k = blk * 8 + j;
            if (k >= rd.draws) break;  // rd.draws counts chunk draws
            const uint64_t word = o.x[j >> 1];
            const uint32_t x = (j & 1) ? (uint32_t)(word >> 32) : (uint32_t)word;
            const uint64_t first = rd.slice_off + (x % nchunks) * kSampleChunk;
            const uint64_t count = min((uint64_t)kSampleChunk, end - first);
            chunks[rd.draw_off + k] = first | (count << 32);
        }
    }
}

// One warp per sampled chunk of the draw range [d0, d1): coalesced loads of its edges, each hooked.
template <bool kCheck>
__global__ void cc_sample_hook(uint32_t *par, const uint32_t *__restrict__ u, const uint32_t *__restrict__ v,
                               const uint64_t *__restrict__ chunks, uint64_t d0, uint64_t d1, uint32_t n,
                               uint32_t *err) {
    pdl_wait();
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t d = d0 + (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); d < d1; d += warps) {
        const uint64_t c = chunks[d];
        if (lane < (uint32_t)(c >> 32)) {
            const uint64_t e = (c & 0xFFFFFFFFull) + lane;
            edge_hook_checked<kCheck>(par, __ldg(u + e), __ldg(v + e), n, err);
        }
    }
}

__global__ void cc_compress(uint32_t *par, uint32_t lo, uint32_t hi) {
    pdl_wait();
    for (uint32_t i = lo + blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += gridDim.x * blockDim.x)
        par[i] = find_root_ro(par, i);
}

// Full compression, 4 consecutive vertices per thread: one 16-byte load of their parents, then
// the grandparents of all four requested together (most chains end there), then the rare longer
// chains; one 16-byte store. Only roots are written, as in cc_compress.
__global__ void cc_compress4(uint32_t *par, uint32_t n4) {
    pdl_wait();
    uint4 *p4 = reinterpret_cast<uint4 *>(par);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x) {
        const uint4 p = p4[i];
        const uint32_t v0 = 4 * i;
        uint32_t r0 = p.x, r1 = p.y, r2 = p.z, r3 = p.w;
        const uint32_t g0 = r0 != v0 ? par[r0] : r0, g1 = r1 != v0 + 1 ? par[r1] : r1;
        const uint32_t g2 = r2 != v0 + 2 ? par[r2] : r2, g3 = r3 != v0 + 3 ? par[r3] : r3;
        r0 = g0 == r0 ? r0 : find_root_ro(par, g0);
        r1 = g1 == r1 ? r1 : find_root_ro(par, g1);
        r2 = g2 == r2 ? r2 : find_root_ro(par, g2);
        r3 = g3 == r3 ? r3 : find_root_ro(par, g3);
        if (r0 != p.x || r1 != p.y || r2 != p.z || r3 != p.w) p4[i] = make_uint4(r0, r1, r2, r3);
    }
}

// Compression of [0, n): the vectorised body over whole 4-vertex groups, the scalar kernel for
// the tail (the parent array is 256-byte aligned).
void compress_all(cac_ctx *ctx, uint32_t *par, uint32_t n, cudaStream_t s);

// The end of the sampling round in one launch: full compression, the giant component and its
// membership bitmap. Every CTA (kGiantSample threads) first finds the giant itself, from the
// roots of the same kGiantSample vertices (fixed spread of positions): every warp finds the mode
// of its 32 samples (__match_any_sync groups equal roots; ties to the smaller root), each of those
// 32 candidates is counted over all samples with shared atomics, and the candidate with the
// largest count wins (ties: the smaller root). The walks only read and no hook runs during this
// kernel, so every CTA sees the same roots and picks the same giant. The choice only decides which
// edges the filter can drop, never the labels. Then its warps take 32-vertex words: each lane walks its vertex to the root,
// writes the root back when it differs (only roots are written, as in cc_compress4), and the
// warp's ballot of (root == giant) is the word. CTA 0 records the giant for the next kernels.
__global__ void __launch_bounds__(kGiantSample) cc_compress_giant_bitmap(uint32_t *par, uint32_t n, uint32_t *giant,
                                                                         uint32_t *bits) {
    pdl_wait();
    __shared__ uint32_t cand[kGiantSample / 32], cnt[kGiantSample / 32];
    __shared__ unsigned long long best;
    const uint32_t i = threadIdx.x, lane = i & 31, w = i >> 5;
    const uint32_t r = find_root_ro(par, (uint32_t)(((uint64_t)i * 2654435761u) % n));
    const uint32_t same = __match_any_sync(0xffffffffu, r);
    const uint32_t c = __popc(same);
    const uint32_t top = __reduce_max_sync(0xffffffffu, c);
    const uint32_t lo = __reduce_max_sync(0xffffffffu, c == top ? 0xFFFFFFFFu - r : 0u);
    if (lane == 0) {
        cand[w] = 0xFFFFFFFFu - lo;
        cnt[w] = 0;
    }
    if (i == 0) best = 0;
    __syncthreads();
#pragma unroll 8
    for (uint32_t k = 0; k < kGiantSample / 32; k++)
        if (r == cand[k]) atomicAdd(&cnt[k], 1u);
    __syncthreads();
    if (i < kGiantSample / 32)
        atomicMax(&best, ((unsigned long long)cnt[i] << 32) | (0xFFFFFFFFu - cand[i]));
    __syncthreads();
    const uint32_t g = 0xFFFFFFFFu - (uint32_t)(best & 0xFFFFFFFFu);
    if (blockIdx.x == 0 && i == 0) *giant = g;
    const uint64_t nw = ((uint64_t)n + 31) / 32;
    const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t wd = ((uint64_t)blockIdx.x * blockDim.x + i) >> 5; wd < nw; wd += warps) {
        const uint64_t x = wd * 32 + lane;
        bool in = false;
        if (x < n) {
            const uint32_t p = par[x];
            const uint32_t root = p == (uint32_t)x ? p : find_root_ro(par, p);
            if (root != p) par[x] = root;
            in = root == g;
        }
        const uint32_t word = __ballot_sync(0xffffffffu, in);
        if (lane == 0) bits[wd] = word;
    }
}

// Closing pass without a sampling round: every edge hooks, 4 edges per thread step through
// 16-byte streaming loads.
template <bool kVec, bool kCheck>
__global__ void __launch_bounds__(kThreads) cc_edge_pass(uint32_t *par, const uint32_t *__restrict__ u,
                                                         const uint32_t *__restrict__ v, uint64_t m, uint32_t n,
                                                         uint32_t *err) {
    pdl_wait();
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
            edge_hook_checked<kCheck>(par, a.x, b.x, n, err);
            edge_hook_checked<kCheck>(par, a.y, b.y, n, err);
            edge_hook_checked<kCheck>(par, a.z, b.z, n, err);
            edge_hook_checked<kCheck>(par, a.w, b.w, n, err);
        }
        done = m4 << 2;
    }
    for (uint64_t e = done + tid; e < m; e += stride)
        edge_hook_checked<kCheck>(par, __ldcs(u + e), __ldcs(v + e), n, err);
}

// Filter pass after the sampling round (the reference's slice rewrite that drops loops,
// IteratedSparseSampling.hpp:160-172): a pure streaming read of every edge; edges with both
// endpoints in the giant component are dropped, the others are appended to this CTA's region of
// `surv` (region = the CTA's contiguous range of 256-edge tiles, so no global counter is
// contended). A warp owns a tile: lane l reads edges 4l..4l+3 and 128+4l..128+4l+3 of it with
// two fully coalesced 512-byte loads per endpoint array, keeps 8 edges in flight, and appends its
// survivors after one warp scan and one shared-memory atomic. The membership bitmap's first
// `swords` words are staged in shared memory, the rest read through the read-only path.
template <bool kAllSmem, bool kCheck>
__global__ void __launch_bounds__(kEdgeThreads) cc_filter(const uint32_t *__restrict__ u,
                                                          const uint32_t *__restrict__ v, uint64_t tiles,
                                                          const uint32_t *__restrict__ gbits, uint32_t nwords,
                                                          uint2 *__restrict__ surv, uint32_t *__restrict__ counts,
                                                          uint32_t n, uint32_t *err) {
    pdl_wait();
    extern __shared__ uint32_t sbits[];
    __shared__ uint32_t s_n;
    const uint32_t swords = min(nwords, (uint32_t)kSmemBitmapWords);
    for (uint32_t i = threadIdx.x; i < swords; i += blockDim.x) sbits[i] = gbits[i];
    if (threadIdx.x == 0) s_n = 0;
    __syncthreads();
    const uint64_t per = (tiles + gridDim.x - 1) / gridDim.x;
    const uint64_t t0 = min(tiles, (uint64_t)blockIdx.x * per), t1 = min(tiles, t0 + per);
    uint2 *out = surv + t0 * 256;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    auto in_giant = [&](uint32_t x) -> bool {
        const uint32_t w = x >> 5;
        const uint32_t word = (kAllSmem || w < swords) ? sbits[w] : __ldg(gbits + w);
        return (word >> (x & 31)) & 1u;
    };
    const uint4 *u4 = reinterpret_cast<const uint4 *>(u);
    const uint4 *v4 = reinterpret_cast<const uint4 *>(v);
    auto process = [&](const uint4 &ua, const uint4 &ub, const uint4 &va, const uint4 &vb) {
        const uint32_t a[8] = {ua.x, ua.y, ua.z, ua.w, ub.x, ub.y, ub.z, ub.w};
        const uint32_t b[8] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, vb.w};
        uint32_t keep = 0, bad = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const bool ok = !kCheck || (a[k] < n && b[k] < n);  // an invalid edge is neither tested nor kept
            bad |= !ok;
            keep |= (uint32_t)(ok && !(in_giant(ok ? a[k] : 0u) && in_giant(ok ? b[k] : 0u))) << k;
        }
        if (kCheck && bad) atomicOr(err, kErrBadId);
        const uint32_t cnt = __popc(keep);
        uint32_t incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        if (total == 0) return;
        uint32_t base = 0;
        if (lane == 31) base = atomicAdd(&s_n, total);
        base = __shfl_sync(0xffffffffu, base, 31) + incl - cnt;
#pragma unroll
        for (int k = 0; k < 8; k++)
            if ((keep >> k) & 1u) out[base++] = make_uint2(a[k], b[k]);
    };
    // two tiles per warp step: all eight 512-byte loads are issued before either tile is used
    for (uint64_t t = t0 + 2 * (uint64_t)warp; t < t1; t += 2 * (uint64_t)nwarps) {
        const bool two = t + 1 < t1;
        const uint4 z = make_uint4(0, 0, 0, 0);
        const uint4 ua = __ldcs(u4 + t * 64 + lane), ub = __ldcs(u4 + t * 64 + 32 + lane);
        const uint4 va = __ldcs(v4 + t * 64 + lane), vb = __ldcs(v4 + t * 64 + 32 + lane);
        const uint4 uc = two ? __ldcs(u4 + (t + 1) * 64 + lane) : z, ud = two ? __ldcs(u4 + (t + 1) * 64 + 32 + lane) : z;
        const uint4 vc = two ? __ldcs(v4 + (t + 1) * 64 + lane) : z, vd = two ? __ldcs(v4 + (t + 1) * 64 + 32 + lane) : z;
        process(ua, ub, va, vb);
        if (two) process(uc, ud, vc, vd);
    }
    __syncthreads();
    if (threadIdx.x == 0) counts[blockIdx.x] = s_n;
}

// Union of the surviving edges (the reference's next round on the remaining slice). Regions of
// the filter CTAs are addressed through the prefix of their counts.
__global__ void __launch_bounds__(kThreads) cc_hook_survivors(uint32_t *par, const uint2 *__restrict__ surv,
                                                              const uint32_t *__restrict__ counts, uint32_t nregions,
                                                              uint64_t region_stride) {
    pdl_wait();
    __shared__ uint32_t pre[kMaxRegions + 1];
    __shared__ uint32_t wsum[kThreads / 32];
    static_assert(kMaxRegions == 4 * kThreads, "four region counts per thread");
    // exclusive prefix of the region counts: four per thread, then a block scan of the sums
    uint32_t c[4], local = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const uint32_t r = 4 * threadIdx.x + k;
        c[k] = r < nregions ? counts[r] : 0;
        local += c[k];
    }
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    uint32_t before = 0;
    for (uint32_t w = 0; w < warp; w++) before += wsum[w];
    uint32_t acc = before + incl - local;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const uint32_t r = 4 * threadIdx.x + k;
        if (r <= nregions) pre[r] = acc;
        acc += c[k];
    }
    if (threadIdx.x == kThreads - 1 && nregions == kMaxRegions) pre[kMaxRegions] = acc;
    __syncthreads();
    const uint32_t total = pre[nregions];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = nregions - 1;  // last region whose first survivor <= i
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (pre[mid] <= i) lo = mid; else hi = mid - 1;
        }
        const uint2 e = surv[(uint64_t)lo * region_stride + (i - pre[lo])];
        edge_hook(par, e.x, e.y);
    }
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
    pdl_wait();
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
    pdl_wait();
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
    pdl_wait();
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
    pdl_wait();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t r = par[i];
        if (r != i) labels[i] = labels[r];
    }
}

// CTAs of cc_compress_giant_bitmap: two per SM (kGiantSample threads each), fewer for small n.
unsigned giant_grid(cac_ctx *ctx, uint32_t n) {
    const uint64_t words = ((uint64_t)n + 31) / 32;
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((words + 31) / 32, (uint64_t)ctx->num_sms * 2));
}

int grid_for(cac_ctx *ctx, uint64_t work, int per_sm) {
    const uint64_t need = (work + kThreads - 1) / kThreads;
    const uint64_t cap = (uint64_t)ctx->num_sms * per_sm;
    return (int)std::max<uint64_t>(1, std::min(need, cap));
}

void compress_all(cac_ctx *ctx, uint32_t *par, uint32_t n, cudaStream_t s) {
    const uint32_t n4 = n / 4;
    if (n4) launch_pdl(cc_compress4, grid_for(ctx, n4, 8), kThreads, 0, s, par, n4);
    if (n & 3) launch_pdl(cc_compress, 1, 32, 0, s, par, 4 * n4, n);
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

size_t cc_scratch_bytes(uint32_t n, uint32_t ranks, uint64_t m) {
    const size_t ntiles = ((size_t)n + kTile - 1) / kTile;
    const size_t nwords = ((size_t)n + 31) / 32;
    return align_up((size_t)n * 4) + 2 * align_up(ntiles * 4 + 4) + align_up(256) +
           align_up(sizeof(RankDesc) * (size_t)ranks) + align_up(nwords * 4 + 4) + align_up(kMaxRegions * 4) +
           align_up((m + 4 * (uint64_t)kMaxRegions) * 8);
}

namespace {

// Everything one query enqueues, resolved on the host.
struct CCLaunch {
    uint32_t n = 0;
    uint64_t m = 0;
    const uint32_t *u = nullptr, *v = nullptr;
    uint32_t *labels = nullptr;
    uint32_t ranks = 1;
    uint32_t *par = nullptr, *counts = nullptr, *offsets = nullptr, *total = nullptr, *giant = nullptr;
    uint32_t *bits = nullptr, *region_counts = nullptr;
    uint2 *surv = nullptr;
    RankDesc *d_ranks = nullptr;
    const RankDesc *h_ranks = nullptr;
    uint32_t ntiles = 0, nwords = 0;
    uint64_t blocks = 0, draws = 0, drawn = 0;  // sitmo blocks, chunk draws, sampled edges
    uint64_t *chunks = nullptr;                  // per draw: first edge | count << 32
    uint32_t *err = nullptr;                     // total + kErrWord
    bool vec = false;
    bool check = false;                          // endpoints not validated: every kernel checks them
};

int record(cac_ctx *ctx, int i, bool capturing) {
    if (capturing) CAC_CUDA_TRY(cudaEventRecordWithFlags(ctx->ev[i], ctx->stream, cudaEventRecordExternal));
    else CAC_CUDA_TRY(cudaEventRecord(ctx->ev[i], ctx->stream));
    return CAC_OK;
}

// Enqueues the whole query on the ctx stream (directly, or into a graph being captured).
int cc_enqueue(cac_ctx *ctx, const CCLaunch &L, bool capturing) {
    cudaStream_t s = ctx->stream;
    const uint32_t n = L.n;
    const uint64_t m = L.m;
    CAC_TRY(record(ctx, 0, capturing));
    CAC_CUDA_TRY(cudaMemsetAsync(L.err, 0, 4, s));
    CAC_CUDA_TRY(launch_pdl(cc_init, grid_for(ctx, n, 8), kThreads, 0, s, L.par, n));
    if (L.draws > 0 && m > 0) {
        CAC_CUDA_TRY(cudaMemcpyAsync(L.d_ranks, L.h_ranks, sizeof(RankDesc) * L.ranks, cudaMemcpyHostToDevice, s));
        // The draws are hooked in the slices of kSliceEighths: forest building from singletons is
        // the expensive part of CC, and flattening the trees between slices keeps the union walks
        // of the next slice one or two hops long. (Drawing inside the hooking CTAs instead of in
        // one kernel up front measured slower: the rank search and the block cipher then sit on
        // every slice's critical path.)
        CAC_CUDA_TRY(launch_pdl(cc_sample_draws, grid_for(ctx, L.blocks, 8), kThreads, 0, s,
                                static_cast<const RankDesc *>(L.d_ranks), (int)L.ranks, L.blocks, L.chunks));
        constexpr uint32_t sub = sizeof(kSliceEighths) / sizeof(kSliceEighths[0]);
        uint32_t eighths = 0;
        for (uint32_t k = 0; k < sub; k++) {
            const uint64_t d0 = L.draws * eighths / 8;
            eighths += kSliceEighths[k];
            const uint64_t d1 = L.draws * eighths / 8;
            if (d1 > d0) {
                auto hook = L.check ? cc_sample_hook<true> : cc_sample_hook<false>;
                CAC_CUDA_TRY(launch_pdl(hook, grid_for(ctx, (d1 - d0) * 32, 8), kThreads, 0, s, L.par, L.u, L.v,
                                        static_cast<const uint64_t *>(L.chunks), d0, d1, n, L.err));
            }
            if (k + 1 < sub) compress_all(ctx, L.par, n, s);
        }
        CAC_CUDA_TRY(launch_pdl(cc_compress_giant_bitmap, giant_grid(ctx, n), kGiantSample, 0, s, L.par, n, L.giant,
                                L.bits));
    }
    CAC_TRY(record(ctx, 1, capturing));
    if (m > 0) {
        if (L.draws > 0) {
            // a sampling round ran, so a giant component exists: filter, then hook the survivors
            const size_t sm = (size_t)std::min(L.nwords, kSmemBitmapWords) * 4;
            const uint64_t tiles = L.vec ? m >> 8 : 0;  // 256-edge tiles; the rest goes to the scalar pass
            const uint32_t regions = (uint32_t)std::max<uint64_t>(
                1, std::min<uint64_t>({(uint64_t)ctx->num_sms, (uint64_t)kMaxRegions, tiles}));
            const uint64_t per = (tiles + regions - 1) / regions;
            if (tiles) {
                auto filt = L.nwords <= kSmemBitmapWords ? (L.check ? cc_filter<true, true> : cc_filter<true, false>)
                                                         : (L.check ? cc_filter<false, true> : cc_filter<false, false>);
                CAC_CUDA_TRY(launch_pdl(filt, regions, kEdgeThreads, sm, s, L.u, L.v, tiles,
                                        static_cast<const uint32_t *>(L.bits), L.nwords, L.surv, L.region_counts, n,
                                        L.err));
            }
            CAC_TRY(record(ctx, 4, capturing));
            if (tiles)
                CAC_CUDA_TRY(launch_pdl(cc_hook_survivors, (unsigned)ctx->num_sms * kSurvivorBlocksPerSm, kThreads, 0, s,
                                        L.par, static_cast<const uint2 *>(L.surv),
                                        static_cast<const uint32_t *>(L.region_counts), regions, per * 256));
            const uint64_t done = tiles * 256;
            if (done < m)
                (L.check ? cc_edge_pass<false, true> : cc_edge_pass<false, false>)<<<grid_for(ctx, m - done, 8), kThreads,
                                                                                       0, s>>>(
                    L.par, L.u + done, L.v + done, m - done, n, L.err);
        } else {
            const int grid = grid_for(ctx, (m + 3) / 4, 8);
            auto pass = L.vec ? (L.check ? cc_edge_pass<true, true> : cc_edge_pass<true, false>)
                              : (L.check ? cc_edge_pass<false, true> : cc_edge_pass<false, false>);
            pass<<<grid, kThreads, 0, s>>>(L.par, L.u, L.v, m, n, L.err);
            CAC_TRY(record(ctx, 4, capturing));
        }
    } else {
        CAC_TRY(record(ctx, 4, capturing));
    }
    CAC_TRY(record(ctx, 2, capturing));
    // (A single-pass count and rank by decoupled look-back measured slower: BA n=1,024,000 20.4 vs
    // 18.5 us, R-MAT scale 22 48.6 vs 34.0 us for the labelling.)
    CAC_CUDA_TRY(launch_pdl(cc_finalize_count, L.ntiles, kThreads, 0, s, L.par, n, L.counts));
    CAC_CUDA_TRY(launch_pdl(cc_scan_tiles, 1, 1024, 0, s, static_cast<const uint32_t *>(L.counts), L.offsets, L.ntiles,
                            L.total));
    if (L.labels) {
        CAC_CUDA_TRY(launch_pdl(cc_rank_roots, L.ntiles, kThreads, 0, s, static_cast<const uint32_t *>(L.par), n,
                                static_cast<const uint32_t *>(L.offsets), L.labels));
        CAC_CUDA_TRY(launch_pdl(cc_label_all, grid_for(ctx, n, 8), kThreads, 0, s,
                                static_cast<const uint32_t *>(L.par), n, L.labels));
    }
    CAC_CUDA_TRY(cudaGetLastError());
    CAC_CUDA_TRY(cudaMemcpyAsync(ctx->pinned_u32, L.total, (kErrWord + 1) * 4, cudaMemcpyDeviceToHost, s));
    CAC_TRY(record(ctx, 3, capturing));
    return CAC_OK;
}

// The query's error word, copied back with its count.
int check_ids_word(cac_ctx *ctx, uint32_t n) {
    if (ctx->pinned_u32[kErrWord] & kErrBadId) {
        set_error("connected components: an edge endpoint is >= n = " + std::to_string(n) +
                  " (such edges were skipped; the labels are not valid)");
        return CAC_ERR_INVALID;
    }
    return CAC_OK;
}

bool same_key(const CCGraphKey &a, const CCGraphKey &b) {
    return a.u == b.u && a.v == b.v && a.labels == b.labels && a.n == b.n && a.m == b.m && a.seed == b.seed &&
           a.ranks == b.ranks && a.arena_base == b.arena_base && a.arena_cap == b.arena_cap && a.check == b.check;
}

}  // namespace

void cc_graph_reset(cac_ctx *ctx) {
    if (ctx->cc_exec) cudaGraphExecDestroy(ctx->cc_exec);
    ctx->cc_exec = nullptr;
    ctx->cc_key = CCGraphKey{};
    if (ctx->cc_stream_exec) cudaGraphExecDestroy(ctx->cc_stream_exec);
    ctx->cc_stream_exec = nullptr;
    ctx->cc_stream_key = CCStreamKey{};
}

int cc_run(cac_ctx *ctx, uint32_t n, uint64_t m, const uint32_t *d_u, const uint32_t *d_v, uint32_t seed,
           uint32_t ranks, uint32_t *d_labels, cac_cc_result *res, bool check_ids) {
    if (ranks == 0) ranks = 1;
    cudaStream_t s = ctx->stream;
    if (n == 0) {
        if (res) *res = cac_cc_result{};
        return CAC_OK;
    }
    const CCPlan plan = cc_plan(n, m, ranks);
    uint64_t chunk_slots = 1;
    for (uint32_t r = 0; r < ranks; r++) chunk_slots += (plan.draws[r] + kSampleChunk - 1) / kSampleChunk;
    CCLaunch L;
    L.n = n;
    L.m = m;
    L.u = d_u;
    L.v = d_v;
    L.labels = d_labels;
    L.ranks = ranks;
    L.ntiles = (uint32_t)(((uint64_t)n + kTile - 1) / kTile);
    L.nwords = (uint32_t)(((uint64_t)n + 31) / 32);
    L.vec = ((reinterpret_cast<uintptr_t>(d_u) | reinterpret_cast<uintptr_t>(d_v)) & 15) == 0;
    L.check = check_ids;

    CAC_TRY(arena_reserve(ctx, cc_scratch_bytes(n, ranks, m) + align_up(chunk_slots * 8)));
    arena_reset(ctx);
    L.par = (uint32_t *)arena_take(ctx, (size_t)n * 4);
    L.counts = (uint32_t *)arena_take(ctx, (size_t)L.ntiles * 4 + 4);
    L.offsets = (uint32_t *)arena_take(ctx, (size_t)L.ntiles * 4 + 4);
    L.total = (uint32_t *)arena_take(ctx, 256);
    L.giant = L.total + 8;
    L.err = L.total + kErrWord;
    L.d_ranks = (RankDesc *)arena_take(ctx, sizeof(RankDesc) * ranks);
    L.bits = (uint32_t *)arena_take(ctx, (size_t)L.nwords * 4 + 4);
    L.region_counts = (uint32_t *)arena_take(ctx, kMaxRegions * 4);
    L.surv = (uint2 *)arena_take(ctx, (m + 4 * (uint64_t)kMaxRegions) * 8);
    L.chunks = (uint64_t *)arena_take(ctx, chunk_slots * 8);

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
    for (uint32_t r = 0; r < ranks; r++) {
        const uint64_t chunk_draws = (plan.draws[r] + kSampleChunk - 1) / kSampleChunk;
        hr[r].slice_off = plan.slice_off[r];
        hr[r].slice_len = plan.slice_len[r];
        hr[r].draws = chunk_draws;
        hr[r].block_off = L.blocks;
        hr[r].draw_off = L.draws;
        hr[r].key0 = seed + r;
        hr[r].pad = 0;
        L.blocks += (chunk_draws + 7) / 8;
        L.draws += chunk_draws;
        L.drawn += chunk_draws * kSampleChunk;
    }
    L.h_ranks = hr;
    if (L.draws > 0 && m > 0) {
        CAC_TRY(smem_optin(ctx, cc_filter<true, true>));
        CAC_TRY(smem_optin(ctx, cc_filter<false, true>));
        CAC_TRY(smem_optin(ctx, cc_filter<true, false>));
        CAC_TRY(smem_optin(ctx, cc_filter<false, false>));
    }

    // Repeated identical queries replay a captured CUDA graph: one launch instead of a dozen
    // kernel launches and copies. The first sighting of a key runs directly; the second captures.
    CCGraphKey key{d_u, d_v, d_labels, n, m, seed, ranks, ctx->arena.base, ctx->arena.cap, check_ids};
    if (!pinned) {
        cc_graph_reset(ctx);
        CAC_TRY(cc_enqueue(ctx, L, false));
    } else if (same_key(key, ctx->cc_key) && ctx->cc_exec) {
        CAC_CUDA_TRY(cudaGraphLaunch(ctx->cc_exec, s));
    } else if (same_key(key, ctx->cc_key)) {
        cudaGraph_t graph = nullptr;
        CAC_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        const int st = cc_enqueue(ctx, L, true);
        const cudaError_t ce = cudaStreamEndCapture(s, &graph);
        if (st != CAC_OK) {
            if (graph) cudaGraphDestroy(graph);
            return st;
        }
        CAC_CUDA_TRY(ce);
        const cudaError_t ie = cudaGraphInstantiate(&ctx->cc_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            ctx->cc_exec = nullptr;
            cudaGetLastError();
            CAC_TRY(cc_enqueue(ctx, L, false));
        } else {
            CAC_CUDA_TRY(cudaGraphLaunch(ctx->cc_exec, s));
        }
    } else {
        cc_graph_reset(ctx);
        ctx->cc_key = key;
        CAC_TRY(cc_enqueue(ctx, L, false));
    }
    CAC_CUDA_TRY(cudaStreamSynchronize(s));
    CAC_TRY(check_ids_word(ctx, n));
    if (res) {
        res->num_components = ctx->pinned_u32[0];
        res->rounds = (L.draws > 0 ? 1u : 0u) + (m > 0 ? 1u : 0u);  // sampling round + closing pass
        res->sampled_edges = L.drawn;
        CAC_CUDA_TRY(cudaEventElapsedTime(&res->device_ms, ctx->ev[0], ctx->ev[3]));
        CAC_CUDA_TRY(cudaEventElapsedTime(&res->edge_pass_ms, ctx->ev[1], ctx->ev[4]));
        CAC_CUDA_TRY(cudaEventElapsedTime(&res->sample_ms, ctx->ev[0], ctx->ev[1]));
        CAC_CUDA_TRY(cudaEventElapsedTime(&res->hook_ms, ctx->ev[4], ctx->ev[2]));
        CAC_CUDA_TRY(cudaEventElapsedTime(&res->label_ms, ctx->ev[2], ctx->ev[3]));
    }
    return CAC_OK;
}

// Device address of a pinned (page-locked, mapped) host array, or null for pageable memory.
static const uint32_t *pinned_device_view(const uint32_t *h) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? static_cast<const uint32_t *>(a.devicePointer) : nullptr;
}

// Connected components of an edge list that is still in host memory (cac_cc_edges). The
// host-to-device link (about 209 GB/s on a GB300 host, measured for copy-engine copies and for
// kernels reading pinned host memory alike) is the bound: BA n=1,024,000 needs 0.63 ms to cross it
// and 0.23 ms to solve once resident. So the edges cross in an order that lets the ctx stream do
// its work behind the copy:
//   1. kStreamPieces evenly spaced pieces, together as large as the reference's sample budget
//      (edgesToSamplePerProcessor: n^1.045 * 1.2 edges), land first: pulled by one kernel from
//      pinned host arrays while the copy engine starts on the gaps, else as one strided copy per
//      array. They are hooked piece by piece, one edge per thread, with a full compression after
//      each: this is the sampling round (the pieces are spread over the whole list, so an edge list
//      sorted by vertex still yields a sample of the whole graph).
//   2. The giant component of the sample is fixed as a bitmap.
//   3. The gaps between the pieces cross on the copy stream, each streamed through the filter as
//      it lands: edges with both ends in the giant component are dropped, the others hooked.
// What is left after the last byte arrives is one gap's filter and the labelling. Labels -- rank
// of each component's smallest vertex -- are the same as cc_run's for any edge order and sample.
// h_labels (optional) receives the labels before the call returns. A repeated call with the same
// buffers replays the whole sequence as one captured CUDA graph.
namespace {

// Everything one streamed query enqueues, resolved on the host.
struct StreamLaunch {
    uint32_t n = 0;
    uint64_t m = 0;
    const uint32_t *h_u = nullptr, *h_v = nullptr;  // host edge arrays (copy-engine source)
    const uint32_t *z_u = nullptr, *z_v = nullptr;  // their device views when pinned and aligned, else null
    uint32_t *d_u = nullptr, *d_v = nullptr, *d_labels = nullptr, *h_labels = nullptr;
    uint32_t *par = nullptr, *counts = nullptr, *offsets = nullptr, *total = nullptr, *giant = nullptr;
    uint32_t *bits = nullptr, *region_counts = nullptr;
    uint2 *surv = nullptr;
    uint32_t ntiles = 0, nwords = 0;
    bool vec = false, filtered = false;
    std::vector<std::pair<uint64_t, uint64_t>> parts;  // (first edge, count): pieces, then gaps
};

// Copies the sample pieces of a pinned host edge list into the device arrays: kernel loads of
// pinned host memory cross the link at the copy engine's rate, and one launch moves all pieces
// (the copy engine would take one copy per piece and array). Piece i is the 16-byte words
// [i * seg4, i * seg4 + piece4) of each array.
__global__ void cc_pull_pieces(const uint4 *__restrict__ hu, const uint4 *__restrict__ hv, uint4 *__restrict__ du,
                               uint4 *__restrict__ dv, uint64_t seg4, uint64_t piece4, uint32_t pieces) {
    pdl_wait();
    const uint64_t total = piece4 * pieces;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = k / piece4, x = i * seg4 + (k - i * piece4);
        const uint4 a = hu[x], b = hv[x];
        du[x] = a;
        dv[x] = b;
    }
}

int stream_enqueue(cac_ctx *ctx, const StreamLaunch &L, bool capturing) {
    cudaStream_t s = ctx->stream;
    const uint32_t n = L.n;
    CAC_TRY(record(ctx, 0, capturing));
    cc_init<<<grid_for(ctx, n, 8), kThreads, 0, s>>>(L.par, n);
    CAC_CUDA_TRY(cudaMemsetAsync(L.total + kErrWord, 0, 4, s));
    // the copies start after everything already queued on the ctx stream (the staging buffers
    // may still be read by the previous query)
    cudaEvent_t *ev = ctx->chunk_ev;
    CAC_CUDA_TRY(cudaEventRecord(ev[0], s));
    CAC_CUDA_TRY(cudaStreamWaitEvent(ctx->copy_stream, ev[0], 0));
    // The pieces land first: pulled by a kernel on the ctx stream from pinned host arrays (the
    // copy engine meanwhile starts on the gaps), else as one strided copy per array ahead of the
    // gaps on the copy stream.
    const uint64_t seg = L.filtered ? L.parts[1].first : 0, piece = L.filtered ? L.parts[0].second : 0;
    if (L.filtered && L.z_u) {
        cc_pull_pieces<<<grid_for(ctx, piece / 4 * kStreamPieces, 8), kThreads, 0, s>>>(
            reinterpret_cast<const uint4 *>(L.z_u), reinterpret_cast<const uint4 *>(L.z_v),
            reinterpret_cast<uint4 *>(L.d_u), reinterpret_cast<uint4 *>(L.d_v), seg / 4, piece / 4, kStreamPieces);
    } else if (L.filtered) {
        CAC_CUDA_TRY(cudaMemcpy2DAsync(L.d_u, seg * 4, L.h_u, seg * 4, piece * 4, kStreamPieces,
                                       cudaMemcpyHostToDevice, ctx->copy_stream));
        CAC_CUDA_TRY(cudaMemcpy2DAsync(L.d_v, seg * 4, L.h_v, seg * 4, piece * 4, kStreamPieces,
                                       cudaMemcpyHostToDevice, ctx->copy_stream));
        CAC_CUDA_TRY(cudaEventRecord(ev[1], ctx->copy_stream));
    }
    for (size_t c = L.filtered ? kStreamPieces : 0; c < L.parts.size(); c++) {
        const uint64_t e0 = L.parts[c].first, len = L.parts[c].second;
        CAC_CUDA_TRY(cudaMemcpyAsync(L.d_u + e0, L.h_u + e0, len * 4, cudaMemcpyHostToDevice, ctx->copy_stream));
        CAC_CUDA_TRY(cudaMemcpyAsync(L.d_v + e0, L.h_v + e0, len * 4, cudaMemcpyHostToDevice, ctx->copy_stream));
        CAC_CUDA_TRY(cudaEventRecord(ev[1 + c], ctx->copy_stream));
    }
    for (size_t c = 0; c < L.parts.size(); c++) {
        const uint64_t e0 = L.parts[c].first, len = L.parts[c].second;
        // a part copied by the copy engine is waited for (the strided piece copy: before piece 0)
        if (!L.filtered || c >= kStreamPieces || (c == 0 && !L.z_u)) CAC_CUDA_TRY(cudaStreamWaitEvent(s, ev[1 + c], 0));
        if (!L.filtered || c < kStreamPieces) {
            // a piece of the sample (or, unfiltered, a chunk): every edge hooks, one edge per
            // thread (union walks are latency chains, so more of them run at once), then the
            // trees are flattened so the next part's walks stay one or two hops long
            cc_edge_pass<false, true><<<grid_for(ctx, len, 8), kThreads, 0, s>>>(L.par, L.d_u + e0, L.d_v + e0, len, n,
                                                                           L.total + kErrWord);
            if (L.filtered && c + 1 == kStreamPieces) {
                cc_compress_giant_bitmap<<<giant_grid(ctx, n), kGiantSample, 0, s>>>(L.par, n, L.giant, L.bits);
                CAC_TRY(record(ctx, 1, capturing));
            } else if (c + 1 < L.parts.size()) {
                compress_all(ctx, L.par, n, s);
            }
        } else {
            const uint64_t tiles = len >> 8;  // 256-edge tiles; the rest goes to the scalar pass
            const uint32_t regions = (uint32_t)std::max<uint64_t>(
                1, std::min<uint64_t>({(uint64_t)ctx->num_sms, (uint64_t)kMaxRegions, tiles}));
            const uint64_t tper = (tiles + regions - 1) / regions;
            if (tiles) {
                const size_t sm = (size_t)std::min(L.nwords, kSmemBitmapWords) * 4;
                auto filt = L.nwords <= kSmemBitmapWords ? cc_filter<true, true> : cc_filter<false, true>;
                filt<<<regions, kEdgeThreads, sm, s>>>(L.d_u + e0, L.d_v + e0, tiles, L.bits, L.nwords, L.surv,
                                                       L.region_counts, n, L.total + kErrWord);
                cc_hook_survivors<<<(unsigned)ctx->num_sms * kSurvivorBlocksPerSm, kThreads, 0, s>>>(L.par, L.surv, L.region_counts,
                                                                                   regions, tper * 256);
            }
            const uint64_t done = tiles * 256;
            if (done < len)
                cc_edge_pass<false, true><<<grid_for(ctx, len - done, 8), kThreads, 0, s>>>(
                    L.par, L.d_u + e0 + done, L.d_v + e0 + done, len - done, n, L.total + kErrWord);
        }
    }
    if (!L.filtered) CAC_TRY(record(ctx, 1, capturing));
    CAC_TRY(record(ctx, 2, capturing));
    cc_finalize_count<<<L.ntiles, kThreads, 0, s>>>(L.par, n, L.counts);
    cc_scan_tiles<<<1, 1024, 0, s>>>(L.counts, L.offsets, L.ntiles, L.total);
    if (L.d_labels) {
        cc_rank_roots<<<L.ntiles, kThreads, 0, s>>>(L.par, n, L.offsets, L.d_labels);
        cc_label_all<<<grid_for(ctx, n, 8), kThreads, 0, s>>>(L.par, n, L.d_labels);
    }
    CAC_CUDA_TRY(cudaGetLastError());
    CAC_CUDA_TRY(cudaMemcpyAsync(ctx->pinned_u32, L.total, (kErrWord + 1) * 4, cudaMemcpyDeviceToHost, s));
    CAC_TRY(record(ctx, 3, capturing));
    if (L.d_labels && L.h_labels)
        CAC_CUDA_TRY(cudaMemcpyAsync(L.h_labels, L.d_labels, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
    return CAC_OK;
}

bool same_stream_key(const CCStreamKey &a, const CCStreamKey &b) {
    return a.h_u == b.h_u && a.h_v == b.h_v && a.h_labels == b.h_labels && a.d_u == b.d_u && a.d_v == b.d_v &&
           a.d_labels == b.d_labels && a.n == b.n && a.m == b.m && a.zero_copy == b.zero_copy &&
           a.arena_base == b.arena_base && a.arena_cap == b.arena_cap;
}

}  // namespace

int cc_run_streamed(cac_ctx *ctx, uint32_t n, uint64_t m, const uint32_t *h_u, const uint32_t *h_v, uint32_t *d_u,
                    uint32_t *d_v, uint32_t *d_labels, uint32_t *h_labels, cac_cc_result *res) {
    cudaStream_t s = ctx->stream;
    if (res) *res = cac_cc_result{};
    if (n == 0) return CAC_OK;
    if (!ctx->copy_stream) {
        CAC_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
        for (auto &e : ctx->chunk_ev) CAC_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    StreamLaunch L;
    L.n = n;
    L.m = m;
    L.h_u = h_u;
    L.h_v = h_v;
    L.d_u = d_u;
    L.d_v = d_v;
    L.d_labels = d_labels;
    L.h_labels = h_labels;
    L.ntiles = (uint32_t)(((uint64_t)n + kTile - 1) / kTile);
    L.nwords = (uint32_t)(((uint64_t)n + 31) / 32);
    L.vec = ((reinterpret_cast<uintptr_t>(d_u) | reinterpret_cast<uintptr_t>(d_v)) & 15) == 0;
    // Segment i of the list is [i * seg, (i + 1) * seg), the last one running to m; its piece is
    // the first `piece` edges, its gap the rest. seg and piece are multiples of 256 edges, so
    // every piece and gap starts 1 KB aligned and all but the last gap are whole filter tiles.
    const uint64_t budget = std::min<uint64_t>(m, (uint64_t)(std::pow((float)n, 1.0f + 0.09f / 2) * (1.0f + 0.2f)));
    const uint64_t seg = (m / kStreamPieces) & ~255ull;
    const uint64_t piece = seg ? std::min<uint64_t>(seg, ((budget + kStreamPieces - 1) / kStreamPieces + 255) & ~255ull)
                               : 0;
    L.filtered = L.vec && seg > 0;
    const uint64_t max_gap = L.filtered ? m - (kStreamPieces - 1) * seg - piece : 0;
    CAC_TRY(arena_reserve(ctx, align_up((size_t)n * 4) + 2 * align_up((size_t)L.ntiles * 4 + 4) + align_up(256) +
                                   (L.filtered ? align_up((size_t)L.nwords * 4 + 4) + align_up(kMaxRegions * 4) +
                                                     align_up((max_gap + 4 * (uint64_t)kMaxRegions) * 8)
                                               : 0)));
    arena_reset(ctx);
    L.par = (uint32_t *)arena_take(ctx, (size_t)n * 4);
    L.counts = (uint32_t *)arena_take(ctx, (size_t)L.ntiles * 4 + 4);
    L.offsets = (uint32_t *)arena_take(ctx, (size_t)L.ntiles * 4 + 4);
    L.total = (uint32_t *)arena_take(ctx, 256);
    L.giant = L.total + 8;
    if (L.filtered) {
        L.bits = (uint32_t *)arena_take(ctx, (size_t)L.nwords * 4 + 4);
        L.region_counts = (uint32_t *)arena_take(ctx, kMaxRegions * 4);
        L.surv = (uint2 *)arena_take(ctx, (max_gap + 4 * (uint64_t)kMaxRegions) * 8);
        CAC_TRY(smem_optin(ctx, cc_filter<true, true>));
        CAC_TRY(smem_optin(ctx, cc_filter<false, true>));
        CAC_TRY(smem_optin(ctx, cc_filter<true, false>));
        CAC_TRY(smem_optin(ctx, cc_filter<false, false>));
        // pinned, 16-byte aligned host arrays: the pieces are pulled by a kernel
        L.z_u = pinned_device_view(h_u);
        L.z_v = pinned_device_view(h_v);
        if (!L.z_u || !L.z_v || ((reinterpret_cast<uintptr_t>(L.z_u) | reinterpret_cast<uintptr_t>(L.z_v)) & 15))
            L.z_u = L.z_v = nullptr;
        for (uint32_t i = 0; i < kStreamPieces; i++) L.parts.push_back({i * seg, piece});
        for (uint32_t i = 0; i < kStreamPieces; i++) {
            const uint64_t g0 = i * seg + piece, g1 = (i + 1 == kStreamPieces) ? m : (i + 1) * seg;
            if (g1 > g0) L.parts.push_back({g0, g1 - g0});
        }
    } else if (m) {
        // no filter: the whole list in kStreamPieces chunks with 16-byte aligned starts
        const uint64_t per = ((m + kStreamPieces - 1) / kStreamPieces + 1023) & ~1023ull;
        for (uint64_t e0 = 0; e0 < m; e0 += per) L.parts.push_back({e0, std::min(per, m - e0)});
    }

    // A repeated identical call replays a captured CUDA graph, as cc_run does: the first sighting
    // of a key runs directly, the second captures.
    CCStreamKey key{h_u, h_v, h_labels, d_u, d_v, d_labels, n, m, L.z_u != nullptr, ctx->arena.base, ctx->arena.cap};
    if (same_stream_key(key, ctx->cc_stream_key) && ctx->cc_stream_exec) {
        CAC_CUDA_TRY(cudaGraphLaunch(ctx->cc_stream_exec, s));
    } else if (same_stream_key(key, ctx->cc_stream_key)) {
        cudaGraph_t graph = nullptr;
        CAC_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        const int st = stream_enqueue(ctx, L, true);
        const cudaError_t ce = cudaStreamEndCapture(s, &graph);
        if (st != CAC_OK) {
            if (graph) cudaGraphDestroy(graph);
            return st;
        }
        CAC_CUDA_TRY(ce);
        const cudaError_t ie = cudaGraphInstantiate(&ctx->cc_stream_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            ctx->cc_stream_exec = nullptr;
            cudaGetLastError();
            CAC_TRY(stream_enqueue(ctx, L, false));
        } else {
            CAC_CUDA_TRY(cudaGraphLaunch(ctx->cc_stream_exec, s));
        }
    } else {
        if (ctx->cc_stream_exec) cudaGraphExecDestroy(ctx->cc_stream_exec);
        ctx->cc_stream_exec = nullptr;
        ctx->cc_stream_key = key;
        CAC_TRY(stream_enqueue(ctx, L, false));
    }
    CAC_CUDA_TRY(cudaStreamSynchronize(s));
    CAC_TRY(check_ids_word(ctx, n));
    if (res) {
        res->num_components = ctx->pinned_u32[0];
        res->rounds = (L.filtered ? 1u : 0u) + (m > 0 ? 1u : 0u);  // sample pieces + streamed gaps
        res->sampled_edges = L.filtered ? kStreamPieces * piece : 0;
        CAC_CUDA_TRY(cudaEventElapsedTime(&res->device_ms, ctx->ev[0], ctx->ev[3]));
        CAC_CUDA_TRY(cudaEventElapsedTime(&res->sample_ms, ctx->ev[0], ctx->ev[1]));
        CAC_CUDA_TRY(cudaEventElapsedTime(&res->edge_pass_ms, ctx->ev[1], ctx->ev[2]));
        CAC_CUDA_TRY(cudaEventElapsedTime(&res->label_ms, ctx->ev[2], ctx->ev[3]));
    }
    return CAC_OK;
}

}  // namespace cac

// ---------------------------------------------------------------------------------------------
// Allocation-free connected components (cac_cc_noalloc).
//
// Some callers cannot allocate device memory: a plugin running inside a host framework whose
// device memory is owned by that framework's allocator, or a latency-bound serving path that
// must not take cudaMalloc's implicit synchronisation. For them this entry point runs the
// single-pass form of the CC query (hook every edge, compress, count, label) with all of its
// scratch in one file-scope device array of fixed size, so it performs no device allocation of
// its own. The array belongs to this module: every GPU that loads the library holds it (16 MiB
// for the parent array plus 33 KiB of tile counters and offsets) until the process exits.
namespace cac {
namespace {

constexpr uint32_t kNoAllocMaxVertices = 1u << 22;  // 4,194,304 vertices
constexpr uint32_t kNoAllocMaxTiles = (kNoAllocMaxVertices + kTile - 1) / kTile;
constexpr int kNoAllocMaxDevices = 64;

struct NoAllocScratch {
    uint32_t parent[kNoAllocMaxVertices];
    uint32_t counts[kNoAllocMaxTiles + 1];
    uint32_t offsets[kNoAllocMaxTiles + 1];
    uint32_t total[64];
};

__device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// The component count, or 0xFFFFFFFF when an edge endpoint was >= n (the edge was skipped).
__global__ void cc_noalloc_count(const uint32_t *total, uint32_t *out) {
    pdl_wait();
    *out = total[kErrWord] ? 0xFFFFFFFFu : total[0];
}

// Per-device set-up, with that device current: the device address of the scratch array (its
// host-side name is only a stand-in) and the SM count used to size the grids. A device counts as
// set up only once both succeeded, so a call that failed here (for instance one made while its
// stream was being captured, when the module may still have to be loaded) is retried in full by
// the next call instead of failing for the rest of the process.
struct NoAllocDevice {
    std::mutex mu;
    bool ready = false;
    NoAllocScratch *scratch = nullptr;
    int sms = 0;
};
NoAllocDevice g_noalloc_devices[kNoAllocMaxDevices];

cudaError_t noalloc_setup(NoAllocDevice &D, int dev) {
    std::lock_guard<std::mutex> lock(D.mu);
    if (D.ready) return cudaSuccess;
    void *p = nullptr;
    int sms = 0;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) {
        cudaGetLastError();  // not sticky: the next call tries again
        return e;
    }
    D.scratch = reinterpret_cast<NoAllocScratch *>(p);
    D.sms = sms;
    D.ready = true;
    return cudaSuccess;
}

}  // namespace
}  // namespace cac

extern "C" int cac_cc_noalloc(uint32_t n, uint64_t m, const uint32_t *u_dev, const uint32_t *v_dev,
                              uint32_t *labels_dev, uint32_t *num_components_dev, void *stream) {
    using namespace cac;
    if (n > kNoAllocMaxVertices) {
        set_error("cac_cc_noalloc: n = " + std::to_string(n) + " exceeds the allocation-free limit of " +
                  std::to_string(kNoAllocMaxVertices) + " vertices; use cac_cc for larger graphs");
        return CAC_ERR_INVALID;
    }
    if (m > 0xFFFFFFFFull || (m && (!u_dev || !v_dev))) {
        set_error("cac_cc_noalloc: invalid edge arrays (m must be < 2^32 and u/v non-null when m > 0)");
        return CAC_ERR_INVALID;
    }
    int dev = 0;
    CAC_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) {
        set_error("cac_cc_noalloc: device ordinal " + std::to_string(dev) + " out of range");
        return CAC_ERR_INVALID;
    }
    NoAllocDevice &D = g_noalloc_devices[dev];
    const cudaError_t se = noalloc_setup(D, dev);
    if (se != cudaSuccess) {
        set_error(std::string("cac_cc_noalloc: scratch set-up failed (the call may be retried): ") +
                  cudaGetErrorString(se));
        return CAC_ERR_CUDA;
    }
    cudaStream_t s = (cudaStream_t)stream;
    NoAllocScratch *S = D.scratch;
    auto grid = [&](uint64_t work) {
        return (int)std::max<uint64_t>(1, std::min<uint64_t>((work + kThreads - 1) / kThreads, (uint64_t)D.sms * 8));
    };
    if (n == 0) {
        // no vertices: 0 components, or 0xFFFFFFFF when there are edges (every endpoint is >= n)
        if (num_components_dev) CAC_CUDA_TRY(cudaMemsetAsync(num_components_dev, m ? 0xFF : 0, 4, s));
        return CAC_OK;
    }
    // Nothing in the scratch needs to start at zero: parent[] is initialised by cc_init, the tile
    // counters and the total are fully written before they are read.
    const uint32_t ntiles = (uint32_t)(((uint64_t)n + kTile - 1) / kTile);
    cc_init<<<grid(n), kThreads, 0, s>>>(S->parent, n);
    CAC_CUDA_TRY(cudaMemsetAsync(S->total + kErrWord, 0, 4, s));
    if (m > 0) {
        const bool vec = ((reinterpret_cast<uintptr_t>(u_dev) | reinterpret_cast<uintptr_t>(v_dev)) & 15) == 0;
        if (vec) cc_edge_pass<true, true><<<grid((m + 3) / 4), kThreads, 0, s>>>(S->parent, u_dev, v_dev, m, n,
                                                                                 S->total + kErrWord);
        else cc_edge_pass<false, true><<<grid(m), kThreads, 0, s>>>(S->parent, u_dev, v_dev, m, n, S->total + kErrWord);
    }
    cc_finalize_count<<<ntiles, kThreads, 0, s>>>(S->parent, n, S->counts);
    cc_scan_tiles<<<1, 1024, 0, s>>>(S->counts, S->offsets, ntiles, S->total);
    if (labels_dev) {
        cc_rank_roots<<<ntiles, kThreads, 0, s>>>(S->parent, n, S->offsets, labels_dev);
        cc_label_all<<<grid(n), kThreads, 0, s>>>(S->parent, n, labels_dev);
    }
    if (num_components_dev) cc_noalloc_count<<<1, 1, 0, s>>>(S->total, num_components_dev);
    CAC_CUDA_TRY(cudaGetLastError());
    return CAC_OK;
}
