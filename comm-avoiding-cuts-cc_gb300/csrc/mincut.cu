// Minimum cut: the GB300 form of the reference's square_root low-concurrency trial loop
// (src/SquareRootCut.cpp:86-148) with every trial of every virtual rank in flight at once.
//
// One trial (virtual rank r, index i) = the reference's SequentialSquareRootCut::compute
// (src/SequentialSquareRootCut.cpp:4-67) followed by one Karger-Stein trial
// (src/karger-stein/co_mincut.h:176-223):
//   Stage 1  iss_shrink_kernel, one CTA per trial: rounds of (vertex count) weighted draws over
//            the edges that are not loops, contracted in draw order by a shared-memory union-find
//            until t = min(n, ceil(2 sqrt(m) + 1)) vertices remain; vertices renamed to the rank
//            of their smallest member.
//   Stage 2  dense_build_kernel: the t x t adjacency matrix of the contracted graph in HBM
//            (u64 entries, global atomics per edge).
//   Stage 3  Karger-Stein, level-synchronous over all trials of a wave:
//              prep_rows_kernel / prefix_rows_kernel  row sums + 32-column block prefixes of every
//                                                     matrix that is contracted this level
//              contract_kernel   one CTA per child: draws (row by binary search over row prefixes,
//                                column by block prefix + a 32-entry scan), contraction in draw
//                                order until max(ceil(n/sqrt 2)+1, 128) vertices, labels by rank
//                                of the smallest member, member lists by counting sort
//              quotient_warp_kernel / quotient_shared_row_kernel
//                                the child's matrix: member rows summed, every column added into
//                                its label's slot of the output row in shared memory (integer
//                                atomics); a warp per output row, or a CTA's 8 warps on one row at
//                                large N (autotuned per size bucket)
//              sw_leaf_kernel    one 128-thread CTA per leaf (n <= 128), a thread per vertex:
//                                Stoer-Wagner maximum-adjacency
//                                phases with Nagamochi-Ono-Ibaraki contractions on the matrix held
//                                in shared memory (circulant half storage); atomicMin into the
//                                trial's cut
// The random stream of every draw is addressed by (seed + r, i, tag, 0) and (round, draw index),
// tag 1 for Stage 1 and 1 + h for the Karger-Stein child with heap index h, so a CPU replay of
// the same trial reproduces it bit for bit (oracle/mincut.c).
#include "cac_internal.h"
#include "sitmo.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <type_traits>

namespace cac {
namespace {

constexpr uint32_t kSharedRowMinN = 2000;  // before tuning: quotient steps from this N on use the shared-row kernel
constexpr uint32_t kSharedRows = 8;         // output rows per CTA of the shared-row quotient

constexpr uint32_t kMaxSmemVertices = kMaxDenseVertices;  // union-find of a contraction held in shared memory
constexpr int kBatch = 1024;                  // draws gathered before the ordered contraction
constexpr int kNT = 512;                      // threads of the per-trial / per-task CTAs
constexpr uint32_t kDropped = 0xFFFFFFFFu;    // task whose source matrix has no edges left
constexpr uint64_t kU64Max = 0xFFFFFFFFFFFFFFFFull;

// Stage 1 of one trial: its graph, its contraction target and its stream key, its scratch.
struct ShrinkDesc {
    const uint32_t *U, *V, *W;
    uint64_t m;
    uint64_t *pre;     // m: inclusive prefix of the non-loop weights
    uint32_t *lab;     // n: output labels (rank of the smallest member)
    uint32_t *k_out;   // output: number of vertices left
    uint32_t n, target;
    uint32_t k0, idx;  // stream key words 0, 1: seed + virtual rank, trial index within the rank
};

// Stage 2 of one trial: scatter its (relabelled) edges into its k x k matrix.
struct DenseDesc {
    const uint32_t *U, *V, *W;
    const uint32_t *lab;  // nullable: identity
    void *mat;            // k x k, u32 entries when `small`, else u64
    uint64_t m;
    uint32_t k, small;
    // planned ahead: k is the trial's target, checked against Stage 1's own count before any write
    const uint32_t *k_act = nullptr;
    uint32_t *err = nullptr;
};

struct SrcDesc {
    const void *mat;      // N x N row-major, u32 entries when `small`, else u64
    uint64_t *rowpre;     // N: inclusive prefix of row sums
    uint64_t *blk;        // N x nb: per row, inclusive prefix of 32-column block sums
    uint64_t *cut;        // the trial's cut (root matrices deliver the minimum weighted degree bound)
    uint32_t N, nb;
    uint32_t is_root, small;  // small: the graph's total weight is below 2^32
};

struct TaskDesc {
    uint64_t tag;         // stream key word 2 (1 + heap index)
    uint64_t *cut;        // the trial's cut
    uint32_t *lab;        // N labels (output)
    uint32_t *memb_off;   // k + 1 offsets (output)
    uint32_t *members;    // N vertices grouped by label (output)
    uint32_t src;         // index into the SrcDesc array
    uint32_t target;
    uint32_t round;
    uint32_t k0, idx;     // stream key words 0, 1
    uint32_t pad;         // 1: the graph's total weight is below 2^32 (every entry fits 32 bits)
};

struct LeafDesc {
    const void *mat;          // u32 entries when `small`, else u64
    uint64_t *cut;
    const uint64_t *rowsum;   // the N row sums written with the matrix (a quotient's), or null
    uint32_t N;
    uint32_t small;  // entries fit in 32 bits
};

// Node matrices are stored with u32 entries when the graph's total weight is below 2^32 (every
// entry, row sum and cut of every node fits), else u64.
// Kernels that read or write node matrices are instantiated for one entry width Tm each and
// skip the nodes of the other width; the host launches the u64 instance only when some node of
// the step needs it.
// Row stride of an N x N node matrix: N rounded up to a multiple of 4 entries, so that every row
// starts on a 16-byte boundary (16-byte loads). Entries past column N - 1 are never used.
__host__ __device__ __forceinline__ uint64_t ld_of(uint32_t N) { return ((uint64_t)N + 3) & ~(uint64_t)3; }

template <typename Tm>
__device__ __forceinline__ bool width_is(uint32_t small) {
    return (small != 0) == (sizeof(Tm) == 4);
}

// ---------------------------------------------------------------- block helpers

template <int NT>
__device__ __forceinline__ uint64_t block_excl_scan_u64(uint64_t x, uint64_t &total) {
    __shared__ uint64_t warp_tot[NT / 32];
    const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint64_t s = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(0xffffffffu, s, o);
        if (l >= o) s += y;
    }
    if (l == 31) warp_tot[w] = s;
    __syncthreads();
    if (w == 0) {
        uint64_t t = l < NT / 32 ? warp_tot[l] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (l >= o) t += y;
        }
        if (l < NT / 32) warp_tot[l] = t;
    }
    __syncthreads();
    const uint64_t off = w ? warp_tot[w - 1] : 0;
    total = warp_tot[NT / 32 - 1];
    __syncthreads();
    return off + s - x;
}

template <int NT>
__device__ __forceinline__ uint32_t block_excl_scan_u32(uint32_t x, uint32_t &total) {
    uint64_t t64;
    const uint64_t r = block_excl_scan_u64<NT>(x, t64);
    total = (uint32_t)t64;
    return (uint32_t)r;
}

__device__ __forceinline__ uint32_t sfind(uint32_t *par, uint32_t x) {
    while (par[x] != x) {
        par[x] = par[par[x]];
        x = par[x];
    }
    return x;
}

__device__ __forceinline__ uint32_t sfind_ro(const uint32_t *par, uint32_t x) {
    uint32_t nx;
    while ((nx = par[x]) != x) x = nx;
    return x;
}

// Contract the draw pairs sb[0, nb) into the shared-memory union-find `par` (roots are component
// minima) in draw order until *s_count reaches target -- the sequential rule of the trial.
// With need = count - target links still allowed, the next `need` draws are linked by all threads
// at once (CAS of the larger root onto the smaller, finds without compression): each draw links
// at most once, so the count cannot fall below target, and since draws after the one that reaches
// target link nothing, the partition equals the sequential one. A successful CAS always joins
// two different components, so the number of links is the exact count drop. Repeated until the
// target or the end of the batch; the last few links (need <= 16) are made by thread 0 in draw
// order. Endpoints of linked draws are pointed at their roots after each step.
constexpr uint32_t kSeqTail = 16;

template <int NT>
__device__ void contract_batch(uint32_t *par, const uint2 *sb, uint32_t nb, uint32_t target, uint32_t *s_count,
                               uint32_t *s_nlog) {
    volatile uint32_t *vp = par;
    uint32_t j0 = 0;
    for (;;) {
        __syncthreads();
        const uint32_t c = *s_count;
        if (c <= target || j0 >= nb) break;
        const uint32_t need = c - target;
        if (need <= kSeqTail) {
            if (threadIdx.x == 0) {
                uint32_t cc = c;
                for (uint32_t j = j0; j < nb && cc > target; j++) {
                    const uint32_t x = sfind(par, sb[j].x), y = sfind(par, sb[j].y);
                    if (x != y) {
                        if (x < y) par[y] = x; else par[x] = y;
                        cc--;
                    }
                }
                *s_count = cc;
            }
            __syncthreads();
            break;
        }
        const uint32_t j1 = min(nb, j0 + need);
        if (threadIdx.x == 0) *s_nlog = 0;
        __syncthreads();
        for (uint32_t j = j0 + threadIdx.x; j < j1; j += NT) {
            uint32_t x = sb[j].x, y = sb[j].y;
            for (;;) {
                while (vp[x] != x) x = vp[x];
                while (vp[y] != y) y = vp[y];
                if (x == y) break;
                const uint32_t hi = x > y ? x : y, lo = x > y ? y : x;
                if (atomicCAS(&par[hi], hi, lo) == hi) {
                    atomicAdd(s_nlog, 1u);
                    break;
                }
                x = hi;  // hi was linked meanwhile: find both roots again
                y = lo;
            }
        }
        __syncthreads();
        for (uint32_t j = j0 + threadIdx.x; j < j1; j += NT) {  // point the endpoints at their roots
            const uint32_t x = sb[j].x, y = sb[j].y;
            par[x] = sfind_ro(par, x);
            par[y] = sfind_ro(par, y);
        }
        if (threadIdx.x == 0) *s_count = c - *s_nlog;
        j0 = j1;
    }
    __syncthreads();
}

// first index i in [0, len) with a[i] > y (a non-decreasing, a[len-1] > y)
__device__ __forceinline__ uint64_t upper_bound_u64(const uint64_t *a, uint64_t len, uint64_t y) {
    uint64_t lo = 0, hi = len - 1;
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (a[mid] > y) hi = mid; else lo = mid + 1;
    }
    return lo;
}

// Rank-of-minimum relabel of a compressed min-linked union-find (roots are minima): roots get
// their rank in vertex order, every vertex its root's label. Writes `lab` (global).
template <int NT>
__device__ void rank_labels(const uint32_t *par, uint32_t n, uint32_t *lab) {
    uint32_t off = 0;
    for (uint32_t base = 0; base < n; base += NT) {
        const uint32_t v = base + threadIdx.x;
        const uint32_t f = (v < n && par[v] == v) ? 1u : 0u;
        uint32_t tot;
        const uint32_t r = block_excl_scan_u32<NT>(f, tot);
        if (f) lab[v] = off + r;
        off += tot;
    }
    __syncthreads();
    for (uint32_t v = threadIdx.x; v < n; v += NT) {
        const uint32_t r = par[v];
        if (r != v) lab[v] = lab[r];
    }
    __syncthreads();
}

// ---------------------------------------------------------------- stage 1

// Stage 1 of one trial per CTA. Per round: the weights of the edges that are not loops and their
// inclusive prefix in edge order (warp w owns a contiguous range, its lanes read consecutive
// edges; warp sums, one block-level offset step, then a warp scan per 32 edges writes the
// prefix), a coarse index of the prefix at the end of every `cs`-edge segment in shared memory,
// then (vertex count) draws in batches: each draw finds its segment in the shared index and its
// edge by a short binary search inside the segment, and the batch is contracted in draw order.
constexpr uint32_t kCoarse = 2048;      // Stage 1 coarse prefix index entries (shared memory)
constexpr uint32_t kCoarseRows = 1024;  // contraction: coarse row-prefix index entries (shared memory)

template <int NT>
__global__ void __launch_bounds__(NT) iss_shrink_kernel(const ShrinkDesc *__restrict__ descs) {
    constexpr int NW = NT / 32;
    extern __shared__ __align__(16) unsigned char dsm[];
    uint2 *sb = reinterpret_cast<uint2 *>(dsm);
    uint64_t *coarse = reinterpret_cast<uint64_t *>(dsm + kBatch * sizeof(uint2));
    uint32_t *par = reinterpret_cast<uint32_t *>(dsm + kBatch * sizeof(uint2) + kCoarse * sizeof(uint64_t));
    __shared__ uint32_t s_count, s_nlog;
    __shared__ uint64_t s_w[NW];
    const ShrinkDesc D = descs[blockIdx.x];
    const uint32_t n = D.n, target = D.target;
    const uint64_t m = D.m;
    const uint32_t *__restrict__ U = D.U;
    const uint32_t *__restrict__ V = D.V;
    const uint32_t *__restrict__ Wt = D.W;
    uint64_t *pre = D.pre;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t v = threadIdx.x; v < n; v += NT) par[v] = v;
    if (threadIdx.x == 0) s_count = n;
    __syncthreads();
    const uint64_t wseg = (m + NW - 1) / NW;
    const uint64_t wlo = min(m, (uint64_t)warp * wseg), whi = min(m, wlo + wseg);
    // coarse segments of a multiple of 32 edges, at most kCoarse of them
    const uint64_t cs = max((uint64_t)32, ((m + kCoarse - 1) / kCoarse + 31) / 32 * 32);
    const uint32_t ncs = (uint32_t)((m + cs - 1) / cs);
    for (uint64_t rnd = 0; s_count > target; rnd++) {
        uint64_t wsum = 0;
        for (uint64_t e = wlo + lane; e < whi; e += 32)
            if (par[U[e]] != par[V[e]]) wsum += Wt[e];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) wsum += __shfl_xor_sync(0xffffffffu, wsum, o);
        if (lane == 0) s_w[warp] = wsum;
        __syncthreads();
        uint64_t carry = 0, W = 0;
        for (int i = 0; i < NW; i++) {
            if (i < warp) carry += s_w[i];
            W += s_w[i];
        }
        for (uint64_t e0 = wlo; e0 < whi; e0 += 32) {
            const uint64_t e = e0 + lane;
            uint64_t x = (e < whi && par[U[e]] != par[V[e]]) ? Wt[e] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (e < whi) pre[e] = carry + x;
            carry += __shfl_sync(0xffffffffu, x, 31);
        }
        __syncthreads();
        if (W == 0) break;  // the remaining graph has no edges between its vertices
        for (uint32_t i = threadIdx.x; i < ncs; i += NT) coarse[i] = pre[min(m, (i + 1) * cs) - 1];
        __syncthreads();
        const uint32_t c_start = s_count;
        for (uint32_t base = 0; base < c_start; base += kBatch) {
            const uint32_t nb = min((uint32_t)kBatch, c_start - base);
            for (uint32_t j = threadIdx.x; j < nb; j += NT) {
                const uint64_t y = mulhi64(draw64(D.k0, D.idx, 1, 0, rnd, base + j), W);
                const uint64_t sg = upper_bound_u64(coarse, ncs, y);
                const uint64_t s0 = sg * cs;
                const uint64_t e = s0 + upper_bound_u64(pre + s0, min(cs, m - s0), y);
                sb[j] = make_uint2(U[e], V[e]);
            }
            __syncthreads();
            contract_batch<NT>(par, sb, nb, target, &s_count, &s_nlog);
            if (s_count <= target) break;
        }
        for (uint32_t v = threadIdx.x; v < n; v += NT) par[v] = sfind_ro(par, v);
        __syncthreads();
    }
    rank_labels<NT>(par, n, D.lab);
    if (threadIdx.x == 0) *D.k_out = s_count;
}

// ---------------------------------------------------------------- stage 2

__global__ void dense_build_kernel(const DenseDesc *__restrict__ descs) {
    const DenseDesc D = descs[blockIdx.y];
    if (D.k_act && *D.k_act != D.k) {  // Stage 1 stopped off the target: redo the run
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(D.err, kErrPlan);
        return;
    }
    const uint64_t ldk = ld_of(D.k);
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < D.m; e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t a = D.U[e], b = D.V[e];
        if (D.lab) {
            a = D.lab[a];
            b = D.lab[b];
        }
        if (a == b) continue;
        const uint32_t w = D.W[e];
        if (D.small) {
            atomicAdd(reinterpret_cast<uint32_t *>(D.mat) + (uint64_t)a * ldk + b, w);
            atomicAdd(reinterpret_cast<uint32_t *>(D.mat) + (uint64_t)b * ldk + a, w);
        } else {
            atomicAdd(reinterpret_cast<unsigned long long *>(D.mat) + (uint64_t)a * ldk + b, (unsigned long long)w);
            atomicAdd(reinterpret_cast<unsigned long long *>(D.mat) + (uint64_t)b * ldk + a, (unsigned long long)w);
        }
    }
}

// ---------------------------------------------------------------- stage 3: Karger-Stein

// One warp per matrix row: 32-column block prefixes and the row sum.
template <typename Tm>
__global__ void prep_rows_kernel(const SrcDesc *__restrict__ srcs, const uint64_t *__restrict__ row_off,
                                 uint32_t nsrc, uint64_t total_rows) {
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (gw >= total_rows) return;
    uint32_t lo = 0, hi = nsrc - 1;
    while (lo < hi) {  // last source whose first row <= gw
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (row_off[mid] <= gw) lo = mid; else hi = mid - 1;
    }
    const SrcDesc S = srcs[lo];
    const uint64_t i = gw - row_off[lo];
    if (!width_is<Tm>(S.small)) return;
    const Tm *mat = reinterpret_cast<const Tm *>(S.mat) + i * ld_of(S.N);
    uint64_t run = 0;
    for (uint32_t b0 = 0; b0 < S.nb; b0 += 8) {  // eight 32-column blocks per pass, loads in flight together
        uint64_t x[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const uint32_t j = (b0 + u) * 32 + lane;
            x[u] = (b0 + u < S.nb && j < S.N) ? (uint64_t)__ldg(mat + j) : 0;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int u = 0; u < 8; u++) x[u] += __shfl_xor_sync(0xffffffffu, x[u], o);
        }
#pragma unroll
        for (int u = 0; u < 8; u++) {
            run += x[u];
            if (lane == u && b0 + u < S.nb) S.blk[i * S.nb + b0 + u] = run;
        }
    }
    if (lane == 0) {
        S.rowpre[i] = run;
        if (S.is_root) atomicMin((unsigned long long *)S.cut, (unsigned long long)run);
    }
}

// One CTA per source: row sums -> inclusive prefix (in place).
template <int NT>
__global__ void __launch_bounds__(NT) prefix_rows_kernel(const SrcDesc *__restrict__ srcs) {
    const SrcDesc S = srcs[blockIdx.x];
    uint64_t carry = 0;
    for (uint32_t base = 0; base < S.N; base += NT) {
        const uint32_t i = base + threadIdx.x;
        const uint64_t x = i < S.N ? S.rowpre[i] : 0;
        uint64_t tot;
        const uint64_t ex = block_excl_scan_u64<NT>(x, tot);
        if (i < S.N) S.rowpre[i] = carry + ex + x;
        carry += tot;
    }
}

template <int NT, typename Tm>
__global__ void __launch_bounds__(NT) contract_kernel(const TaskDesc *__restrict__ tasks,
                                                      const SrcDesc *__restrict__ srcs, uint32_t *__restrict__ k_out,
                                                      uint32_t *err) {
    extern __shared__ __align__(16) unsigned char dsm[];
    uint2 *sb = reinterpret_cast<uint2 *>(dsm);
    uint64_t *crow = reinterpret_cast<uint64_t *>(dsm + kBatch * sizeof(uint2));  // coarse row index
    __shared__ uint32_t s_count, s_nlog;
    const TaskDesc T = tasks[blockIdx.x];
    const SrcDesc S = srcs[T.src];
    const uint32_t N = S.N;
    uint32_t *par = reinterpret_cast<uint32_t *>(dsm + kBatch * sizeof(uint2) + kCoarseRows * sizeof(uint64_t));
    uint32_t *cnt = par + N;  // counting-sort counters, N entries
    if (!width_is<Tm>(S.small)) return;
    const Tm *mat = reinterpret_cast<const Tm *>(S.mat);
    const uint64_t W = S.rowpre[N - 1];
    if (W == 0) {  // no edges between the vertices: the cut is 0, nothing to contract
        if (threadIdx.x == 0) {
            k_out[blockIdx.x] = kDropped;
            atomicMin((unsigned long long *)T.cut, 0ull);
        }
        return;
    }
    // row prefix at the end of every `cr`-row segment (every row when N <= kCoarseRows)
    const uint32_t cr = (N + kCoarseRows - 1) / kCoarseRows;
    const uint32_t ncr = (N + cr - 1) / cr;
    for (uint32_t v = threadIdx.x; v < N; v += NT) par[v] = v;
    for (uint32_t i = threadIdx.x; i < ncr; i += NT) crow[i] = S.rowpre[min(N, (i + 1) * cr) - 1];
    if (threadIdx.x == 0) s_count = N;
    __syncthreads();
    for (uint32_t base = 0; base < N; base += kBatch) {
        const uint32_t nb = min((uint32_t)kBatch, N - base);
        for (uint32_t j = threadIdx.x; j < nb; j += NT) {
            const uint64_t y = mulhi64(draw64(T.k0, T.idx, T.tag, 0, T.round, base + j), W);
            // row: first whose inclusive prefix exceeds y (segment in shared memory, then inside it)
            const uint32_t sg = (uint32_t)upper_bound_u64(crow, ncr, y);
            uint32_t a;
            uint64_t before;
            if (cr == 1) {
                a = sg;
                before = a ? crow[a - 1] : 0;
            } else {
                const uint32_t r0 = sg * cr;
                a = r0 + (uint32_t)upper_bound_u64(S.rowpre + r0, min(cr, N - r0), y);
                before = a ? S.rowpre[a - 1] : 0;
            }
            const uint64_t rem = y - before;
            const uint64_t *B = S.blk + (uint64_t)a * S.nb;
            const uint32_t b = (uint32_t)upper_bound_u64(B, S.nb, rem);
            const uint64_t rem2 = rem - (b ? B[b - 1] : 0);
            const uint64_t rb = (uint64_t)a * ld_of(N) + (uint64_t)b * 32;
            const uint32_t lim = min(32u, N - b * 32);
            // column: first whose running sum exceeds rem2, eight entries loaded together per step
            uint64_t acc = 0;
            uint32_t c = lim;
            for (uint32_t c0 = 0; c0 < lim && c == lim; c0 += 8) {
                uint64_t x[8];
#pragma unroll
                for (int k = 0; k < 8; k++) x[k] = c0 + k < lim ? (uint64_t)__ldg(mat + rb + c0 + k) : 0;
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    acc += x[k];
                    if (c == lim && c0 + k < lim && acc > rem2) c = c0 + k;
                }
            }
            if (c >= lim) {  // cannot happen with consistent prefixes; record and clamp
                atomicOr(err, 1u);
                c = lim - 1;
            }
            sb[j] = make_uint2(a, b * 32 + c);
        }
        __syncthreads();
        contract_batch<NT>(par, sb, nb, T.target, &s_count, &s_nlog);
        if (s_count <= T.target) break;
    }
    for (uint32_t v = threadIdx.x; v < N; v += NT) par[v] = sfind_ro(par, v);
    __syncthreads();
    rank_labels<NT>(par, N, T.lab);
    const uint32_t k = s_count;
    // member lists grouped by label (counting sort; order inside a group is irrelevant)
    for (uint32_t l = threadIdx.x; l < k; l += NT) cnt[l] = 0;
    __syncthreads();
    for (uint32_t v = threadIdx.x; v < N; v += NT) atomicAdd(&cnt[T.lab[v]], 1u);
    __syncthreads();
    uint32_t off = 0;
    for (uint32_t base = 0; base < k; base += NT) {
        const uint32_t l = base + threadIdx.x;
        const uint32_t x = l < k ? cnt[l] : 0;
        uint32_t tot;
        const uint32_t ex = block_excl_scan_u32<NT>(x, tot);
        if (l < k) {
            T.memb_off[l] = off + ex;
            cnt[l] = off + ex;  // becomes the scatter cursor
        }
        off += tot;
    }
    if (threadIdx.x == 0) T.memb_off[k] = N;
    __syncthreads();
    for (uint32_t v = threadIdx.x; v < N; v += NT) {
        const uint32_t p = atomicAdd(&cnt[T.lab[v]], 1u);
        T.members[p] = v;
    }
    if (threadIdx.x == 0) k_out[blockIdx.x] = k;
}

__device__ __forceinline__ void sadd(uint32_t *p, uint64_t v) { atomicAdd(p, (uint32_t)v); }
__device__ __forceinline__ void sadd(uint64_t *p, uint64_t v) {
    atomicAdd(reinterpret_cast<unsigned long long *>(p), (unsigned long long)v);
}

// The quotient for large N: one CTA of 8 warps per group of `rows` consecutive output rows, all
// warps on the same output row at a time. The warp kernel below gives every warp its own k-entry
// row in shared memory, which at N in the thousands leaves room for only a few warps per SM; here
// the CTA shares one row (labels + one row: 8 CTAs, 64 warps per SM at N = 4000), and the warps
// split the columns: 128-column chunks (one 16-byte load per lane), chunk c to warp c mod 8, four
// chunks per warp in flight. Per output row: zero the row, sum the member rows chunk by chunk and
// add every column into its label's slot (shared atomics), store the row with the diagonal zeroed
// and its 32-column block sums, then one warp turns the block sums into the block prefixes and the
// row sum (the next step's row prep). Five CTAs per SM (48 registers): measured 1-3% faster on
// K4000 than the four that 60 registers allow.
template <typename Ts, typename Tm>
__global__ void __launch_bounds__(256, 5) quotient_shared_row_kernel(const TaskDesc *__restrict__ tasks,
                                                                  const SrcDesc *__restrict__ srcs,
                                                                  const uint32_t *__restrict__ kdim,
                                                                  const uint64_t *__restrict__ group_task_off,
                                                                  uint32_t ntasks, uint32_t rows,
                                                                  const uint64_t *__restrict__ out_off,
                                                                  unsigned char *out_base, uint32_t lab_words,
                                                                  uint32_t kmax, const uint32_t *__restrict__ kact,
                                                                  uint32_t *err) {
    extern __shared__ __align__(16) unsigned char dsm[];
    const uint64_t gg = blockIdx.x;
    uint32_t lo = 0, hi = ntasks - 1;
    while (lo < hi) {  // last task whose first row group <= gg
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (group_task_off[mid] <= gg) lo = mid; else hi = mid - 1;
    }
    const TaskDesc T = tasks[lo];
    const SrcDesc S = srcs[T.src];
    const uint32_t k = kdim[lo];
    if (kact && kact[lo] != k) {  // planned ahead, and this child stopped off its target: redo the run
        if (threadIdx.x == 0) atomicOr(err, kErrPlan);
        return;
    }
    const uint32_t N = S.N;
    const uint32_t a0 = (uint32_t)(gg - group_task_off[lo]) * rows, a1 = min(k, a0 + rows);
    if (!width_is<Tm>(S.small)) return;
    const Tm *mat = reinterpret_cast<const Tm *>(S.mat);
    constexpr int VEC = 16 / sizeof(Tm);  // columns per 16-byte load
    constexpr uint32_t NWARP = 8;
    using Vec = typename std::conditional<sizeof(Tm) == 4, uint4, ulonglong2>::type;
    const uint64_t ldN = ld_of(N);
    uint32_t *s_lab = reinterpret_cast<uint32_t *>(dsm);  // N
    Ts *qrow = reinterpret_cast<Ts *>(dsm + (size_t)lab_words * 4);  // kmax
    uint64_t *bsum = reinterpret_cast<uint64_t *>(dsm + (size_t)lab_words * 4 + (((size_t)kmax * sizeof(Ts) + 15) & ~(size_t)15));
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) s_lab[i] = T.lab[i];
    Tm *Qt = reinterpret_cast<Tm *>(out_base + out_off[lo]);
    uint64_t *rowsum_out = reinterpret_cast<uint64_t *>(out_base + out_off[ntasks + lo]);
    const uint32_t small = S.small;
    const uint32_t nbk = (k + 31) / 32;
    uint64_t *blk = rowsum_out + k;
    const uint32_t nchunk = (N + 32 * VEC - 1) / (32 * VEC);
    // the row is zeroed once here, then by the output pass of every row as it reads it
    for (uint32_t b = threadIdx.x; b < k; b += blockDim.x) qrow[b] = 0;
    __syncthreads();  // labels staged, row zeroed
    for (uint32_t a = a0; a < a1; a++) {
        const uint32_t p0 = T.memb_off[a], p1 = T.memb_off[a + 1];
        for (uint32_t c0 = warp; c0 < nchunk; c0 += 4 * NWARP) {
            Tm x[4][VEC];
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int t = 0; t < VEC; t++) x[u][t] = 0;
            for (uint32_t p = p0; p < p1; p++) {
                const Vec *row = reinterpret_cast<const Vec *>(mat + (uint64_t)T.members[p] * ldN);
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const uint32_t c = (c0 + u * NWARP) * 32 * VEC + lane * VEC;
                    if (c < N) {
                        const Vec q = __ldg(row + c / VEC);
                        const Tm *e = reinterpret_cast<const Tm *>(&q);
#pragma unroll
                        for (int t = 0; t < VEC; t++) x[u][t] += e[t];
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int t = 0; t < VEC; t++) {
                    const uint32_t j = (c0 + u * NWARP) * 32 * VEC + lane * VEC + t;
                    if (j < N && x[u][t]) sadd(&qrow[s_lab[j]], (uint64_t)x[u][t]);
                }
        }
        __syncthreads();  // the row is complete
        const uint64_t qb = (uint64_t)a * ld_of(k);
        for (uint32_t b0 = warp * 32; b0 < k; b0 += NWARP * 32) {
            const uint32_t b = b0 + lane;
            uint64_t v = (b < k && b != a) ? (uint64_t)qrow[b] : 0;
            if (b < k) {
                Qt[qb + b] = (Tm)v;
                qrow[b] = 0;  // for the next row (the barrier below orders it before that row's adds)
            }
            if (small) {  // every entry < 2^32: two 32-bit reductions of the 16-bit halves are exact
                const uint32_t lo16 = __reduce_add_sync(0xffffffffu, (uint32_t)(v & 0xFFFFu));
                const uint32_t hi16 = __reduce_add_sync(0xffffffffu, (uint32_t)(v >> 16));
                v = (uint64_t)lo16 + ((uint64_t)hi16 << 16);
            } else {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            }
            if (lane == 0) bsum[b0 >> 5] = v;
        }
        __syncthreads();  // block sums complete; the row may be zeroed again after the next barrier
        if (warp == 0) {
            // inclusive prefix of the block sums: lane l owns blocks [l * per, (l + 1) * per)
            const uint32_t per = (nbk + 31) / 32;
            const uint32_t j0 = lane * per, j1 = min(nbk, j0 + per);
            uint64_t own = 0;
            for (uint32_t j = j0; j < j1; j++) own += bsum[j];
            uint64_t incl = own;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint64_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= (uint32_t)o) incl += y;
            }
            uint64_t run = incl - own;
            for (uint32_t j = j0; j < j1; j++) {
                run += bsum[j];
                blk[(uint64_t)a * nbk + j] = run;
            }
            if (lane == 31) rowsum_out[a] = incl;
        }
    }
}

// One CTA per group of `rows` consecutive output rows of one child, one warp per output row at a
// time. The child's labels are staged in shared memory once per CTA. For output row a the warp
// sums the member rows of group a (lanes stride the columns, eight independent loads in flight
// each) and adds every column's sum straight into its label's slot of the warp's output row in
// shared memory (an integer atomic, exact in any order); then it stores the row with the diagonal
// zeroed, and writes the row's 32-column block prefixes and its sum (the next step's row prep).
// Shared memory: the labels, then one k-entry row per warp.
//   Q[a][b] = sum over u in group a, v in group b of A[u][v]
template <typename Ts, typename Tm>
__global__ void __launch_bounds__(256) quotient_warp_kernel(const TaskDesc *__restrict__ tasks,
                                                            const SrcDesc *__restrict__ srcs,
                                                            const uint32_t *__restrict__ kdim,
                                                            const uint64_t *__restrict__ group_task_off,
                                                            uint32_t ntasks, uint32_t rows,
                                                            const uint64_t *__restrict__ out_off,
                                                            unsigned char *out_base, uint32_t lab_words,
                                                            uint32_t kmax, const uint32_t *__restrict__ kact,
                                                            uint32_t *err) {
    // out_off[i]: byte offset of task i's matrix; out_off[ntasks + i]: of its row sums and block
    // prefixes (the next step's row prep)
    extern __shared__ __align__(16) unsigned char dsm[];
    const uint64_t gg = blockIdx.x;
    uint32_t lo = 0, hi = ntasks - 1;
    while (lo < hi) {  // last task whose first row group <= gg
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (group_task_off[mid] <= gg) lo = mid; else hi = mid - 1;
    }
    const TaskDesc T = tasks[lo];
    const SrcDesc S = srcs[T.src];
    const uint32_t k = kdim[lo];
    if (kact && kact[lo] != k) {  // planned ahead, and this child stopped off its target: redo the run
        if (threadIdx.x == 0) atomicOr(err, kErrPlan);
        return;
    }
    const uint32_t N = S.N;
    const uint32_t a0 = (uint32_t)(gg - group_task_off[lo]) * rows, a1 = min(k, a0 + rows);
    if (!width_is<Tm>(S.small)) return;
    const Tm *mat = reinterpret_cast<const Tm *>(S.mat);
    constexpr int VEC = 16 / sizeof(Tm);  // columns per 16-byte load
    using Vec = typename std::conditional<sizeof(Tm) == 4, uint4, ulonglong2>::type;
    const uint64_t ldN = ld_of(N);
    uint32_t *s_lab = reinterpret_cast<uint32_t *>(dsm);  // N
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    // Ts: uint32_t when the graph's total weight is below 2^32 (every entry and row sum fits)
    Ts *qrow = reinterpret_cast<Ts *>(dsm + (size_t)lab_words * 4) + (size_t)warp * kmax;
    for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) s_lab[i] = T.lab[i];
    __syncthreads();
    Tm *Qt = reinterpret_cast<Tm *>(out_base + out_off[lo]);
    uint64_t *rowsum_out = reinterpret_cast<uint64_t *>(out_base + out_off[ntasks + lo]);
    const uint32_t small = S.small;
    const uint32_t nbk = (k + 31) / 32;
    uint64_t *blk = rowsum_out + k;
    // the warp's row is zeroed once here, then by the output pass of every row as it reads it
    for (uint32_t b = lane; b < k; b += 32) qrow[b] = 0;
    __syncwarp();
    for (uint32_t a = a0 + warp; a < a1; a += nw) {
        const uint32_t p0 = T.memb_off[a], p1 = T.memb_off[a + 1];
        // 16-byte loads: lane l reads columns j0 + (32 u + l) VEC .. + VEC - 1 (4 loads per pass);
        // the padding columns of a row are read but never scattered
        for (uint32_t j0 = 0; j0 < N; j0 += 4 * 32 * VEC) {
            Tm x[4][VEC];
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int t = 0; t < VEC; t++) x[u][t] = 0;
            for (uint32_t p = p0; p < p1; p++) {
                const Vec *row = reinterpret_cast<const Vec *>(mat + (uint64_t)T.members[p] * ldN);
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const uint32_t c = j0 + (u * 32 + lane) * VEC;
                    if (c < N) {
                        const Vec q = __ldg(row + c / VEC);
                        const Tm *e = reinterpret_cast<const Tm *>(&q);
#pragma unroll
                        for (int t = 0; t < VEC; t++) x[u][t] += e[t];
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int t = 0; t < VEC; t++) {
                    const uint32_t j = j0 + (u * 32 + lane) * VEC + t;
                    if (j < N && x[u][t]) sadd(&qrow[s_lab[j]], (uint64_t)x[u][t]);
                }
        }
        __syncwarp();
        const uint64_t qb = (uint64_t)a * ld_of(k);
        uint64_t run = 0;
        for (uint32_t b0 = 0; b0 < k; b0 += 128) {  // four 32-column blocks per pass (warp-uniform trip count)
            uint64_t acc[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const uint32_t b = b0 + 32 * u + lane;
                acc[u] = (b < k && b != a) ? (uint64_t)qrow[b] : 0;
                if (b < k) {
                    Qt[qb + b] = (Tm)acc[u];
                    qrow[b] = 0;  // for the next row (the warp barrier after this row orders it)
                }
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                if (small) {  // every entry < 2^32: two 32-bit reductions of the 16-bit halves are exact
                    const uint32_t lo16 = __reduce_add_sync(0xffffffffu, (uint32_t)(acc[u] & 0xFFFFu));
                    const uint32_t hi16 = __reduce_add_sync(0xffffffffu, (uint32_t)(acc[u] >> 16));
                    acc[u] = (uint64_t)lo16 + ((uint64_t)hi16 << 16);
                } else {
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) acc[u] += __shfl_xor_sync(0xffffffffu, acc[u], o);
                }
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                if (b0 + 32 * u < k) {
                    run += acc[u];
                    if (lane == u) blk[(uint64_t)a * nbk + (b0 >> 5) + u] = run;
                }
            }
        }
        if (lane == 0) rowsum_out[a] = run;
        __syncwarp();
    }
}

// ---------------------------------------------------------------- bulk-copy quotient
// The warp-per-row quotient with its member rows staged in shared memory by the bulk-copy (TMA)
// engine instead of loaded into registers: every warp walks its stream of (output row a, member u)
// pairs; while it adds row u of the source into its label slots from shared memory, the copy
// engine already fetches the next member row into the warp's other buffer (one 1-D
// cp.async.bulk per row, completion counted on an mbarrier per buffer). So a warp always has a
// whole row in flight, and its registers hold no row data. Rows start on 16-byte boundaries (ld_of
// pads every row to 4 entries) and their length is a multiple of 16 bytes, as the bulk copy needs.
// Every wait on an mbarrier is bounded: when the bound is reached the kernel sets bit 1 of the
// engine's error word, waits (bounded again) for the copies it still has in flight and returns.
constexpr uint32_t kBulkSpin = 1u << 20;  // bound on one mbarrier wait (polls with a short sleep)

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// lane 0: one bulk copy of `bytes` from global `src` into shared `dst`, completing on `bar`
__device__ __forceinline__ void bulk_row(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// wait until the barrier's phase `parity` has completed; false when the bound ran out
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    for (uint32_t i = 0; i < kBulkSpin; i++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        __nanosleep(32);
    }
    return false;
}

template <typename Ts, typename Tm>
__global__ void __launch_bounds__(256) quotient_bulk_kernel(const TaskDesc *__restrict__ tasks,
                                                            const SrcDesc *__restrict__ srcs,
                                                            const uint32_t *__restrict__ kdim,
                                                            const uint64_t *__restrict__ group_task_off,
                                                            uint32_t ntasks, uint32_t rows,
                                                            const uint64_t *__restrict__ out_off,
                                                            unsigned char *out_base, uint32_t lab_words,
                                                            uint32_t kmax, uint32_t row_words, uint32_t *err,
                                                            const uint32_t *__restrict__ kact) {
    extern __shared__ __align__(16) unsigned char dsm[];  // bulk copies need 16-byte alignment
    const uint64_t gg = blockIdx.x;
    uint32_t lo = 0, hi = ntasks - 1;
    while (lo < hi) {  // last task whose first row group <= gg
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (group_task_off[mid] <= gg) lo = mid; else hi = mid - 1;
    }
    const TaskDesc T = tasks[lo];
    const SrcDesc S = srcs[T.src];
    const uint32_t k = kdim[lo];
    if (kact && kact[lo] != k) {  // planned ahead, and this child stopped off its target: redo the run
        if (threadIdx.x == 0) atomicOr(err, kErrPlan);
        return;
    }
    const uint32_t N = S.N;
    const uint32_t a0 = (uint32_t)(gg - group_task_off[lo]) * rows, a1 = min(k, a0 + rows);
    if (!width_is<Tm>(S.small)) return;
    const Tm *mat = reinterpret_cast<const Tm *>(S.mat);
    constexpr int VEC = 16 / sizeof(Tm);
    using Vec = typename std::conditional<sizeof(Tm) == 4, uint4, ulonglong2>::type;
    const uint64_t ldN = ld_of(N);
    const uint32_t row_bytes = (uint32_t)(ldN * sizeof(Tm));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    // shared memory: 16 mbarriers | labels | per warp: two row buffers, then its k-entry row
    uint64_t *bars = reinterpret_cast<uint64_t *>(dsm);
    uint32_t *s_lab = reinterpret_cast<uint32_t *>(dsm + 128);
    const size_t per_warp = (((size_t)row_words * sizeof(Tm)) * 2 + (size_t)kmax * sizeof(Ts) + 15) & ~(size_t)15;
    unsigned char *wbase = dsm + 128 + (((size_t)lab_words * 4 + 15) & ~(size_t)15) + (size_t)warp * per_warp;
    Tm *const buf0 = reinterpret_cast<Tm *>(wbase);
    Tm *const buf1 = reinterpret_cast<Tm *>(wbase + (size_t)row_words * sizeof(Tm));
    Ts *qrow = reinterpret_cast<Ts *>(wbase + (size_t)row_words * sizeof(Tm) * 2);
    uint64_t *bar = bars + 2 * warp;
    for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) s_lab[i] = T.lab[i];
    if (lane == 0) {
        mbar_init(bar, 1);
        mbar_init(bar + 1, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    Tm *Qt = reinterpret_cast<Tm *>(out_base + out_off[lo]);
    uint64_t *rowsum_out = reinterpret_cast<uint64_t *>(out_base + out_off[ntasks + lo]);
    const uint32_t small = S.small;
    const uint32_t nbk = (k + 31) / 32;
    uint64_t *blk = rowsum_out + k;
    // the warp's stream: rows a = a0 + warp, a0 + warp + nw, ...; members p of each row
    uint32_t a = a0 + warp;
    if (a >= a1) return;  // no row for this warp (its barriers were never armed)
    uint32_t p = T.memb_off[a], pend = T.memb_off[a + 1];
    // per buffer: the phase to wait for next, and whether a copy into it is in flight (bits 0, 1)
    uint32_t parity = 0, inflight = 1;
    bool failed = false;
    if (lane == 0) bulk_row(buf0, mat + (uint64_t)T.members[p] * ldN, row_bytes, bar);
    for (uint32_t b = lane; b < k; b += 32) qrow[b] = 0;
    __syncwarp();
    for (uint32_t item = 0;; item++) {
        const int cur = item & 1, nxt = cur ^ 1;
        // the next item of the stream, fetched while this one is added
        const bool row_done = p + 1 >= pend;
        uint32_t na = a, np = p + 1, npend = pend;
        if (row_done) {
            na = a + nw;
            if (na < a1) {
                np = T.memb_off[na];
                npend = T.memb_off[na + 1];
            }
        }
        const bool has_next = na < a1;
        if (has_next) {
            if (lane == 0) bulk_row(nxt ? buf1 : buf0, mat + (uint64_t)T.members[np] * ldN, row_bytes, bar + nxt);
            inflight |= 1u << nxt;
        }
        if (!mbar_wait(bar + cur, (parity >> cur) & 1u)) {
            failed = true;
            break;
        }
        parity ^= 1u << cur;
        inflight &= ~(1u << cur);
        // add the member row into the label slots of the warp's output row
        const Vec *row = reinterpret_cast<const Vec *>(cur ? buf1 : buf0);
        for (uint32_t c = lane * VEC; c < N; c += 32 * VEC) {
            const Vec q = row[c / VEC];
            const Tm *e = reinterpret_cast<const Tm *>(&q);
#pragma unroll
            for (int t = 0; t < VEC; t++)
                if (c + t < N && e[t]) sadd(&qrow[s_lab[c + t]], (uint64_t)e[t]);
        }
        __syncwarp();  // every lane is done with buf[cur] (it is refilled two items on)
        if (row_done) {
            // row a is complete: store it with the diagonal zeroed, its block prefixes and its sum
            const uint64_t qb = (uint64_t)a * ld_of(k);
            uint64_t run = 0;
            for (uint32_t b0 = 0; b0 < k; b0 += 128) {
                uint64_t acc[4];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const uint32_t b = b0 + 32 * u + lane;
                    acc[u] = (b < k && b != a) ? (uint64_t)qrow[b] : 0;
                    if (b < k) Qt[qb + b] = (Tm)acc[u];
                }
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    if (small) {
                        const uint32_t lo16 = __reduce_add_sync(0xffffffffu, (uint32_t)(acc[u] & 0xFFFFu));
                        const uint32_t hi16 = __reduce_add_sync(0xffffffffu, (uint32_t)(acc[u] >> 16));
                        acc[u] = (uint64_t)lo16 + ((uint64_t)hi16 << 16);
                    } else {
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) acc[u] += __shfl_xor_sync(0xffffffffu, acc[u], o);
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    if (b0 + 32 * u < k) {
                        run += acc[u];
                        if (lane == u) blk[(uint64_t)a * nbk + (b0 >> 5) + u] = run;
                    }
                }
            }
            if (lane == 0) rowsum_out[a] = run;
            __syncwarp();
            for (uint32_t b = lane; b < k; b += 32) qrow[b] = 0;
            __syncwarp();
        }
        if (!has_next) break;
        a = na;
        p = np;
        pend = npend;
    }
    if (failed) {
        if (lane == 0) atomicOr(err, 2u);
        // let the copies still in flight land before the shared memory is released
        for (int b = 0; b < 2; b++)
            if ((inflight >> b) & 1u) mbar_wait(bar + b, (parity >> b) & 1u);
    }
}

// Exact minimum cut of one leaf (n <= 128) by one CTA of 128 threads: maximum-adjacency orderings
// as in the reference's Stoer-Wagner base case (co_mincut_base_case.hpp:52-144), with the
// Nagamochi-Ono-Ibaraki contraction rule (Nagamochi & Ibaraki 1992; Nagamochi, Ono & Ibaraki
// 1994): when vertex w's key reaches q >= lambda while vertex v is scanned, then lambda(v, w) >= q,
// so the edge (v, w) can be contracted without losing any cut below lambda, the best cut value found
// so far (initially the leaf's minimum weighted degree). Every ordering contracts all such
// certified edges plus the last two vertices (the cut of the phase updates lambda), so far fewer
// orderings are needed than the n - 1 of plain Stoer-Wagner; the returned value is the exact
// minimum cut of the leaf.
//   Thread v owns vertex v. A step of an ordering is one warp argmax of (key, smallest vertex), a
//   cross-warp maximum through a double-buffered shared word per warp (one barrier per step), and
//   one key update per thread from the scanned vertex's row. Every certified edge and the pair
//   (second to last, last) joins a vertex to one scanned before it, so when all but the first
//   vertex of the ordering are so joined the leaf contracts to one vertex and the ordering's result
//   is final: a barrier count decides this without building the contraction (the usual case:
//   Karger-Stein leaves of 128 vertices mostly finish in one ordering). Otherwise the pairs are
//   joined by a union-find over vertex slots and the matrix entries are merged pair by pair.
//   Keys stay below 2^56 (total graph weight checked on the host); u32 matrices keep 32-bit keys.
__device__ __forceinline__ uint64_t warp_min_u64(uint64_t x) {
    const uint32_t hi = (uint32_t)(x >> 32);
    const uint32_t top = __reduce_min_sync(0xffffffffu, hi);
    const uint32_t lo = __reduce_min_sync(0xffffffffu, hi == top ? (uint32_t)x : 0xFFFFFFFFu);
    return ((uint64_t)top << 32) | lo;
}

// Circulant half storage of a symmetric N x N matrix with a zero diagonal: row i holds the entries
// (i, (i + d) mod N) for d = 1 .. H, H = floor(N / 2), so every pair is stored once (twice when N
// is even and d = N / 2; both copies are kept equal). A warp reading the entries (x, v) for its
// lanes' v touches consecutive words for the v after x and words H - 1 apart for the v before x,
// so neither half has bank conflicts; a 128-vertex leaf takes half the shared memory of the full
// matrix and twice as many leaves are resident per SM.
__device__ __forceinline__ uint32_t cpos(uint32_t i, uint32_t j, uint32_t N, uint32_t H) {
    const uint32_t d = j >= i ? j - i : j + N - i;
    return d <= H ? i * H + d - 1 : j * H + (N - d) - 1;
}

template <typename Tm>
__device__ __forceinline__ void cset(Tm *M, uint32_t i, uint32_t j, uint32_t N, uint32_t H, Tm val) {
    const uint32_t d = j >= i ? j - i : j + N - i;
    if (d <= H) {
        M[i * H + d - 1] = val;
        if (d == H && !(N & 1u)) M[j * H + H - 1] = val;  // the twin of an even-N antipodal pair
    } else {
        M[j * H + (N - d) - 1] = val;
    }
}

__device__ __forceinline__ uint64_t warp_max_u64(uint64_t x) {
    const uint32_t hi = (uint32_t)(x >> 32);
    const uint32_t top = __reduce_max_sync(0xffffffffu, hi);
    const uint32_t lo = __reduce_max_sync(0xffffffffu, hi == top ? (uint32_t)x : 0u);
    return ((uint64_t)top << 32) | lo;
}

constexpr uint32_t kLeafThreads = 128;

template <typename Tm>
__global__ void __launch_bounds__(kLeafThreads) sw_leaf_kernel(const LeafDesc *__restrict__ leaves) {
    extern __shared__ __align__(16) unsigned char dsm[];
    Tm *M = reinterpret_cast<Tm *>(dsm);
    __shared__ uint8_t uf[128];
    __shared__ uint32_t pairs[128];
    __shared__ uint32_t npairs;
    __shared__ __align__(16) uint64_t wbest[2][4];
    __shared__ __align__(16) uint32_t wbest32[2][4];
    __shared__ uint64_t wsum[4];
    const LeafDesc L = leaves[blockIdx.x];
    const uint32_t N = L.N, H = N / 2;
    const uint32_t v = threadIdx.x, lane = v & 31u, warp = v >> 5;
    // circulant half: thread v loads offset d = v % 64 + 1 of every second row (rows v / 64,
    // v / 64 + 2, ...), eight rows per pass in flight
    {
        const Tm *src = reinterpret_cast<const Tm *>(L.mat);
        const uint64_t ldN = ld_of(N);
        const uint32_t d = (v & 63u) + 1, r0 = v >> 6;
        const bool has = d <= H;
        for (uint32_t i0 = r0; i0 < N; i0 += 16) {
            Tm a[8];
#pragma unroll
            for (int r = 0; r < 8; r++) {
                const uint32_t i = i0 + 2 * r;
                uint32_t j = i + d;
                j = j >= N ? j - N : j;
                a[r] = (i < N && has) ? __ldg(src + (uint64_t)i * ldN + j) : (Tm)0;
            }
#pragma unroll
            for (int r = 0; r < 8; r++) {
                const uint32_t i = i0 + 2 * r;
                if (i < N && has) M[i * H + d - 1] = a[r];
            }
        }
    }
    uf[v] = (uint8_t)v;
    bool active = v < N;
    __syncthreads();
    // lambda starts at the minimum weighted degree (a cut of the leaf): the row sums that came with
    // the matrix, else summed here (row v's own half, then the entries (v - e, v) stored in the rows
    // before it)
    uint64_t deg = kU64Max;
    if (active) {
        if (L.rowsum) {
            deg = __ldg(L.rowsum + v);
        } else {
            deg = 0;
            for (uint32_t e = 1; e <= H; e++) deg += (uint64_t)M[v * H + e - 1];
            for (uint32_t e = 1; e + H < N; e++) deg += (uint64_t)M[(v >= e ? v - e : v + N - e) * H + e - 1];
        }
    }
    {
        const uint64_t wm = warp_min_u64(deg);
        // the degree sum (u32 matrices: every degree below 2^32, summed as two 16-bit halves)
        const uint32_t d = active && deg < (1ull << 32) ? (uint32_t)deg : 0u;
        const uint64_t ws = (uint64_t)__reduce_add_sync(0xffffffffu, d & 0xFFFFu) +
                            ((uint64_t)__reduce_add_sync(0xffffffffu, d >> 16) << 16);
        if (lane == 0) {
            wbest[1][warp] = wm;  // the first step writes wbest[0]
            wsum[warp] = ws;
        }
    }
    __syncthreads();
    uint64_t lambda = wbest[1][0], deg_sum = wsum[0];
    for (int w = 1; w < 4; w++) {
        lambda = wbest[1][w] < lambda ? wbest[1][w] : lambda;
        deg_sum += wsum[w];
    }
    // a key never exceeds the leaf's total weight (half its degree sum, which merges only lower):
    // below 2^24, (key << 8 | 255 - v) is one 32-bit word and the argmax one reduction
    const bool packed32 = sizeof(Tm) == 4 && deg_sum < (1ull << 25);
    using Kt = typename std::conditional<sizeof(Tm) == 4, uint32_t, uint64_t>::type;
    uint32_t cnt = N, par = 0;
    while (cnt > 1) {
        Kt key = 0;
        const Kt lam = lambda > (uint64_t)(Kt)~(Kt)0 ? (Kt)~(Kt)0 : (Kt)lambda;
        bool in_a = false;
        uint32_t mark = 0xFFu;  // vertex to contract into, 0xFF: none
        uint32_t prev = 0, last = 0;
        uint64_t cut_phase = 0;
        for (uint32_t step = 0; step < cnt; step++) {
            const bool elig = active && !in_a;
            uint32_t sv;
            uint64_t top_key;
            if (packed32) {
                const uint32_t wb = __reduce_max_sync(0xffffffffu, elig ? (((uint32_t)key << 8) | (255u - v)) : 0u);
                if (lane == 0) wbest32[par][warp] = wb;
                __syncthreads();
                const uint4 b = *reinterpret_cast<const uint4 *>(&wbest32[par][0]);
                par ^= 1u;
                const uint32_t best = max(max(b.x, b.y), max(b.z, b.w));
                sv = 255u - (best & 255u);
                top_key = best >> 8;
            } else {
            uint64_t wb;  // this warp's best as (key << 8 | 255 - vertex), 0 for none
            if constexpr (sizeof(Tm) == 4) {
                const uint32_t top = __reduce_max_sync(0xffffffffu, elig ? key : 0u);
                const uint32_t vmin = __reduce_min_sync(0xffffffffu, (elig && key == top) ? v : 255u);
                wb = vmin == 255u ? 0 : (((uint64_t)top << 8) | (uint64_t)(255u - vmin));
            } else {
                wb = warp_max_u64(elig ? ((key << 8) | (uint64_t)(255u - v)) : 0);
            }
            if (lane == 0) wbest[par][warp] = wb;
            __syncthreads();
            const ulonglong2 b01 = *reinterpret_cast<const ulonglong2 *>(&wbest[par][0]);
            const ulonglong2 b23 = *reinterpret_cast<const ulonglong2 *>(&wbest[par][2]);
            par ^= 1u;
            const uint64_t m01 = b01.x > b01.y ? b01.x : b01.y, m23 = b23.x > b23.y ? b23.x : b23.y;
            const uint64_t best = m01 > m23 ? m01 : m23;
            sv = 255u - (uint32_t)(best & 255u);
            top_key = best >> 8;
            }
            if (sv >= N) {  // no candidate: cannot happen (cnt - step vertices are unscanned)
                cut_phase = kU64Max;
                break;
            }
            if (step + 1 == cnt) {
                last = sv;
                cut_phase = top_key;
                break;
            }
            in_a = in_a || v == sv;
            prev = sv;
            if (active && !in_a) {
                const Kt c = (Kt)M[cpos(sv, v, N, H)];
                key += c;
                if (c && key >= lam) mark = sv;  // lambda(sv, v) >= key: contractible
            }
        }
        if (cut_phase == kU64Max) break;
        lambda = cut_phase < lambda ? cut_phase : lambda;
        // one vertex left when every vertex but the first of the ordering is joined to an earlier one
        const uint32_t linked = (uint32_t)__syncthreads_count(active && (mark != 0xFFu || v == last));
        if (linked + 1 >= cnt) break;
        // contraction list: (prev, last), then every certified edge (mark[v], v)
        if (v == 0) {
            pairs[0] = (prev << 8) | last;
            npairs = 1;
        }
        __syncthreads();
        if (active && mark != 0xFFu) pairs[atomicAdd(&npairs, 1u)] = (mark << 8) | v;
        __syncthreads();
        // thread 0 joins the pairs' slots (union-find with path halving) and rewrites the list as
        // the (root, root) merges actually made
        if (v == 0) {
            const uint32_t np = npairs;
            uint32_t made = 0;
            for (uint32_t q = 0; q < np && cnt - made > 1; q++) {
                uint32_t x = pairs[q] >> 8, y = pairs[q] & 255u;
                while (uf[x] != x) {
                    uf[x] = uf[uf[x]];
                    x = uf[x];
                }
                while (uf[y] != y) {
                    uf[y] = uf[uf[y]];
                    y = uf[y];
                }
                if (x == y) continue;  // already merged
                uf[y] = (uint8_t)x;
                pairs[made++] = (x << 8) | y;
            }
            npairs = made;
        }
        __syncthreads();
        const uint32_t nm = npairs;
        if (cnt - nm <= 1) break;
        for (uint32_t q = 0; q < nm; q++) {
            const uint32_t x = pairs[q] >> 8, y = pairs[q] & 255u;
            // merge y into x: entry (x, v) += entry (y, v) for every other active v
            if (active && v != x && v != y) {
                const Tm val = M[cpos(x, v, N, H)] + M[cpos(y, v, N, H)];
                cset(M, x, v, N, H, val);
            }
            if (v == y) active = false;
            __syncthreads();
        }
        cnt -= nm;
    }
    if (v == 0) atomicMin((unsigned long long *)L.cut, (unsigned long long)lambda);
}

__global__ void fill_u64(uint64_t *p, uint64_t n, uint64_t value) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = value;
}

// ---------------------------------------------------------------- host orchestration

// Device buffer owned by one call, grown on demand.
struct DevBuf {
    cac_ctx *ctx = nullptr;
    void *p = nullptr;
    size_t cap = 0;
    explicit DevBuf(cac_ctx *c) : ctx(c) {}
    ~DevBuf() { release(); }
    void release() {
        if (p) dev_free(ctx, p, cap);
        p = nullptr;
        cap = 0;
    }
    int ensure(size_t bytes) {
        if (bytes <= cap) return CAC_OK;
        CAC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        release();
        const size_t want = align_up(std::max<size_t>(bytes, 256), 1 << 16);
        CAC_TRY(dev_alloc(ctx, &p, want));
        cap = want;
        return CAC_OK;
    }
    template <typename T> T *as() const { return reinterpret_cast<T *>(p); }
};

// Grow-only scratch buffers kept by the ctx between calls: a fresh device allocation per query
// (cudaMalloc, and a cudaFree that waits for the whole device) cost more than the kernels of a
// small query (admission of square_root on ER(1000, 0.05): 303 us, of which about 100 us of
// kernels). Slots 0..3 belong to the Karger-Stein engine, 4..10 to admission, 11.. to the
// one-shot probes; one engine runs per ctx at a time.
enum ScratchSlot : int {
    kSlotKout, kSlotPrep, kSlotTscratch, kSlotErr, kSlotPre, kSlotLab, kSlotK, kSlotSd, kSlotDd, kSlotSparse,
    kSlotSparseCount, kSlotProbe0, kSlotProbe1, kSlotProbe2, kSlotCount
};

// Descriptor staging of one phase of an engine step: the phase's small host arrays are packed
// (16-byte aligned) into one pinned host buffer and sent with a single copy into one device
// buffer, instead of one pageable copy per array (each a driver call on the host's critical path
// between a step's read-back and its next launches). An event after the copy guards the pinned
// buffer: it is refilled only once its previous copy has run (at once in the usual flow, where
// every step synchronises in its middle).
struct Staging {
    cac_ctx *ctx;
    DevBuf dev;
    unsigned char *host = nullptr;
    size_t hcap = 0, used = 0;
    cudaEvent_t done = nullptr;
    bool pending = false;
    explicit Staging(cac_ctx *c) : ctx(c), dev(c) {}
    Staging(const Staging &) = delete;
    Staging &operator=(const Staging &) = delete;
    ~Staging() {
        if (pending) cudaEventSynchronize(done);
        if (host) cudaFreeHost(host);
        if (done) cudaEventDestroy(done);
    }
    template <typename T> static size_t bytes_of(const std::vector<T> &v) {
        return (sizeof(T) * std::max<size_t>(v.size(), 1) + 15) & ~(size_t)15;
    }
    int begin(size_t bytes) {
        if (!done) CAC_CUDA_TRY(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
        if (pending) {
            CAC_CUDA_TRY(cudaEventSynchronize(done));
            pending = false;
        }
        bytes = std::max<size_t>(bytes, 16);
        if (bytes > hcap) {
            if (host) CAC_CUDA_TRY(cudaFreeHost(host));
            host = nullptr;
            hcap = 0;
            const size_t want = align_up(bytes, 1 << 16);
            CAC_CUDA_TRY(cudaHostAlloc(reinterpret_cast<void **>(&host), want, cudaHostAllocDefault));
            hcap = want;
        }
        CAC_TRY(dev.ensure(bytes));
        used = 0;
        return CAC_OK;
    }
    // copies v into the host buffer; returns where it will be on the device
    template <typename T> T *put(const std::vector<T> &v) {
        const size_t off = used;
        if (!v.empty()) std::memcpy(host + off, v.data(), sizeof(T) * v.size());
        used += bytes_of(v);
        return reinterpret_cast<T *>(static_cast<unsigned char *>(dev.p) + off);
    }
    int flush() {
        if (!used) return CAC_OK;
        CAC_CUDA_TRY(cudaMemcpyAsync(dev.p, host, used, cudaMemcpyHostToDevice, ctx->stream));
        CAC_CUDA_TRY(cudaEventRecord(done, ctx->stream));
        pending = true;
        return CAC_OK;
    }
};

struct CtxScratch {
    std::vector<DevBuf> slots;
    Staging leaf, pre, post;  // an engine step's leaves, then its descriptors before and after its read-back
    explicit CtxScratch(cac_ctx *ctx) : slots(kSlotCount, DevBuf(ctx)), leaf(ctx), pre(ctx), post(ctx) {}
};

CtxScratch &ctx_scratch(cac_ctx *ctx) {
    if (!ctx->ks_scratch) ctx->ks_scratch = new CtxScratch(ctx);
    return *static_cast<CtxScratch *>(ctx->ks_scratch);
}

DevBuf &scratch(cac_ctx *ctx, ScratchSlot slot) { return ctx_scratch(ctx).slots[slot]; }

template <typename T>
int upload(cac_ctx *ctx, DevBuf &buf, const std::vector<T> &v) {
    CAC_TRY(buf.ensure(sizeof(T) * std::max<size_t>(v.size(), 1)));
    if (!v.empty())
        CAC_CUDA_TRY(cudaMemcpyAsync(buf.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, ctx->stream));
    return CAC_OK;
}

size_t leaf_smem(uint32_t N, bool small) { return (size_t)N * (N / 2) * (small ? 4 : 8); }
size_t contract_smem(uint32_t N) { return kBatch * sizeof(uint2) + kCoarseRows * sizeof(uint64_t) + (size_t)2 * N * 4; }

}  // namespace

void ctx_scratch_free(cac_ctx *ctx) {
    delete static_cast<CtxScratch *>(ctx->ks_scratch);
    ctx->ks_scratch = nullptr;
}

// ---- Karger-Stein engine (declared in cac_internal.h) ----

KsEngine::KsEngine(cac_ctx *ctx)
    : ctx_(ctx), d_kout_(&scratch(ctx, kSlotKout)), d_prep_(&scratch(ctx, kSlotPrep)),
      d_tscratch_(&scratch(ctx, kSlotTscratch)), d_err_(&scratch(ctx, kSlotErr)) {}

KsEngine::~KsEngine() {
    cudaStreamSynchronize(ctx_->stream);
    for (const KNode &nd : nodes_) release(nd.buf);
    for (const KTask &t : carried_) release(t.src.buf);
    nodes_.clear();
    carried_.clear();
}

int KsEngine::init_err() {
    DevBuf *e = static_cast<DevBuf *>(d_err_);
    CAC_TRY(e->ensure(4));
    CAC_CUDA_TRY(cudaMemsetAsync(e->p, 0, 4, ctx_->stream));
    return CAC_OK;
}

uint32_t *KsEngine::err_word() const { return static_cast<DevBuf *>(d_err_)->as<uint32_t>(); }

int KsEngine::read_err(uint32_t *err) {
    DevBuf *e = static_cast<DevBuf *>(d_err_);
    *err = 0;
    if (!e->p) return CAC_OK;
    CAC_CUDA_TRY(cudaMemcpyAsync(err, e->p, 4, cudaMemcpyDeviceToHost, ctx_->stream));
    CAC_CUDA_TRY(cudaStreamSynchronize(ctx_->stream));
    return CAC_OK;
}

int engine_error(uint32_t err) {
    if (err & 2u) {
        set_error("Karger-Stein quotient: a bulk-copy wait exceeded its bound");
        return CAC_ERR_TIMEOUT;
    }
    set_error("inconsistent selection prefix in the contraction kernel");
    return CAC_ERR_CUDA;
}

int KsEngine::alloc(size_t bytes, MatBuf **out) {
    *out = nullptr;
    bytes = std::max<size_t>(bytes, 256);
    if (ctx_->budget && ctx_->held + bytes > ctx_->budget) {
        set_error("HBM budget exceeded by a Karger-Stein level buffer of " + std::to_string(bytes) + " bytes");
        return CAC_ERR_OOM;
    }
    void *p = nullptr;
    cudaError_t e = ctx_->pool ? cudaMallocFromPoolAsync(&p, bytes, ctx_->pool, ctx_->stream)
                               : cudaMallocAsync(&p, bytes, ctx_->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error(std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
        return CAC_ERR_OOM;
    }
    ctx_->held += bytes;
    MatBuf *b = new MatBuf{p, bytes, 0};
    *out = b;
    return CAC_OK;
}

void KsEngine::release(MatBuf *b) {
    if (!b) return;
    if (--b->refs > 0) return;
    if (b->refs < 0) {  // released more often than referenced: keep it, report at the next step
        release_err_ = true;
        return;
    }
    if (cudaFreeAsync(b->p, ctx_->stream) != cudaSuccess) {
        cudaGetLastError();  // reported through the engine's error state, not as a sticky CUDA error
        release_err_ = true;
    }
    ctx_->held -= std::min<uint64_t>(ctx_->held, b->bytes);
    delete b;
}

void KsEngine::add(const KNode &nd) {
    nd.buf->refs++;
    nodes_.push_back(nd);
    if (nd.query >= outstanding.size()) outstanding.resize(nd.query + 1, 0);
    outstanding[nd.query]++;
}

int KsEngine::step() {
    cudaStream_t s = ctx_->stream;
    if (release_err_) {
        set_error("Karger-Stein engine: a level buffer was released more often than referenced or could not be freed");
        return CAC_ERR_CUDA;
    }
    DevBuf &d_kout = *static_cast<DevBuf *>(d_kout_), &d_prep = *static_cast<DevBuf *>(d_prep_);
    DevBuf &d_tscratch = *static_cast<DevBuf *>(d_tscratch_);
    uint32_t *d_err = static_cast<DevBuf *>(d_err_)->as<uint32_t>();
    std::vector<MatBuf *> consumed;

    // leaves (n <= 128) -> exact cut; grouped by size and entry width, one launch each
    std::vector<LeafDesc> leaves;
    std::vector<KNode> inner;
    for (const KNode &nd : nodes_) {
        if (nd.N <= 128) {
            if (nd.N >= 2) {
                leaves.push_back(LeafDesc{nd.mat, nd.cut, nd.pre, nd.N, nd.small});
            }
            consumed.push_back(nd.buf);
            outstanding[nd.query]--;
        } else {
            inner.push_back(nd);
        }
    }
    nodes_.clear();
    std::sort(leaves.begin(), leaves.end(),
              [](const LeafDesc &a, const LeafDesc &b) { return a.N != b.N ? a.N > b.N : a.small > b.small; });
    // the leaves, grouped by size and entry width, one launch each (after the descriptor copy)
    auto launch_leaves = [&](const LeafDesc *d_leaves) -> int {
        size_t first = 0;
        while (first < leaves.size()) {
            size_t last = first;
            while (last < leaves.size() && leaves[last].N == leaves[first].N && leaves[last].small == leaves[first].small)
                last++;
            const uint32_t N = leaves[first].N;
            const LeafDesc *dl = d_leaves + first;
            if (leaves[first].small) {
                const size_t sm = leaf_smem(N, true);
                CAC_TRY(smem_optin(ctx_, sw_leaf_kernel<uint32_t>));
                sw_leaf_kernel<uint32_t><<<(unsigned)(last - first), kLeafThreads, sm, s>>>(dl);
            } else {
                const size_t sm = leaf_smem(N, false);
                CAC_TRY(smem_optin(ctx_, sw_leaf_kernel<uint64_t>));
                sw_leaf_kernel<uint64_t><<<(unsigned)(last - first), kLeafThreads, sm, s>>>(dl);
            }
            first = last;
        }
        CAC_CUDA_TRY(cudaGetLastError());
        return CAC_OK;
    };
    Staging &leaf_st = ctx_scratch(ctx_).leaf, &pre_st = ctx_scratch(ctx_).pre, &post_st = ctx_scratch(ctx_).post;
    // the leaves go first: they run while the host plans the step's contractions
    if (!leaves.empty()) {
        CAC_TRY(leaf_st.begin(Staging::bytes_of(leaves)));
        const LeafDesc *dl = leaf_st.put(leaves);
        CAC_TRY(leaf_st.flush());
        CAC_TRY(launch_leaves(dl));
    }

    // sources: inner nodes (two children each) and the matrices of tasks continuing another round
    std::vector<KTask> tasks;
    std::vector<KNode> src_nodes;
    for (const KNode &nd : inner) {
        src_nodes.push_back(nd);
        const uint32_t target = (uint32_t)ks_target((int)nd.N);
        for (uint64_t c = 0; c < 2; c++) tasks.push_back(KTask{nd, 2 * nd.h + c, 0, target, (uint32_t)(src_nodes.size() - 1)});
        outstanding[nd.query]++;  // two tasks replace the node
        consumed.push_back(nd.buf);
    }
    for (KTask t : carried_) {
        src_nodes.push_back(t.src);
        t.src_index = (uint32_t)(src_nodes.size() - 1);
        tasks.push_back(t);
        consumed.push_back(t.src.buf);
    }
    carried_.clear();
    if (tasks.empty()) {
        for (MatBuf *b : consumed) release(b);
        return CAC_OK;
    }
    // sources whose row sums and block prefixes came with their matrix (warp quotient) skip the
    // row prep; the others (roots, large-N quotients) are prepped here from their own list
    std::vector<SrcDesc> srcs(src_nodes.size()), psrcs;
    std::vector<uint64_t> row_off;
    uint64_t rows = 0, prep_elems = 0;
    for (size_t i = 0; i < src_nodes.size(); i++) {
        if (src_nodes[i].pre) continue;
        const uint32_t nb = (src_nodes[i].N + 31) / 32;
        prep_elems += src_nodes[i].N + (uint64_t)src_nodes[i].N * nb;
    }
    CAC_TRY(d_prep.ensure(std::max<uint64_t>(prep_elems, 1) * 8));
    uint64_t pe = 0;
    for (size_t i = 0; i < src_nodes.size(); i++) {
        const KNode &nd = src_nodes[i];
        SrcDesc &S = srcs[i];
        S.mat = nd.mat;
        S.N = nd.N;
        S.nb = (nd.N + 31) / 32;
        S.cut = nd.cut;
        S.is_root = nd.is_root;
        S.small = nd.small;
        if (nd.pre) {
            S.rowpre = nd.pre;
        } else {
            S.rowpre = d_prep.as<uint64_t>() + pe;
            pe += nd.N + (uint64_t)nd.N * S.nb;
            row_off.push_back(rows);
            rows += nd.N;
        }
        S.blk = S.rowpre + nd.N;
        if (!nd.pre) psrcs.push_back(S);
    }

    // contraction of every child
    uint64_t tscratch = 0;
    uint32_t maxN = 0;
    for (const KTask &t : tasks) {
        tscratch += 3 * (uint64_t)t.src.N + 1;
        maxN = std::max(maxN, t.src.N);
    }
    CAC_TRY(d_tscratch.ensure(tscratch * 4));
    std::vector<TaskDesc> td(tasks.size());
    uint64_t ts = 0;
    for (size_t i = 0; i < tasks.size(); i++) {
        const KTask &t = tasks[i];
        TaskDesc &d = td[i];
        d.tag = 1 + t.h;
        d.cut = t.src.cut;
        d.src = t.src_index;
        d.target = t.target;
        d.round = t.round;
        d.k0 = t.src.k0;
        d.idx = t.src.idx;
        d.pad = t.src.small;  // entries (and row sums) below 2^32
        d.lab = d_tscratch.as<uint32_t>() + ts;
        d.members = d.lab + t.src.N;
        d.memb_off = d.members + t.src.N;
        ts += 3 * (uint64_t)t.src.N + 1;
    }
    CAC_TRY(d_kout.ensure(tasks.size() * 4));
    // one descriptor copy for the sources, the row-prep list and the tasks
    CAC_TRY(pre_st.begin(Staging::bytes_of(srcs) + Staging::bytes_of(row_off) + Staging::bytes_of(psrcs) +
                         Staging::bytes_of(td)));
    const SrcDesc *dv_src = pre_st.put(srcs);
    const uint64_t *dv_rowoff = pre_st.put(row_off);
    const SrcDesc *dv_psrc = pre_st.put(psrcs);
    const TaskDesc *dv_task = pre_st.put(td);
    CAC_TRY(pre_st.flush());
    if (rows) {
        bool p32 = false, p64 = false;
        for (const SrcDesc &S : psrcs) (S.small ? p32 : p64) = true;
        const unsigned pg = (unsigned)((rows * 32 + 255) / 256);
        if (p32)
            prep_rows_kernel<uint32_t><<<pg, 256, 0, s>>>(dv_psrc, dv_rowoff, (uint32_t)row_off.size(), rows);
        if (p64)
            prep_rows_kernel<uint64_t><<<pg, 256, 0, s>>>(dv_psrc, dv_rowoff, (uint32_t)row_off.size(), rows);
    }
    prefix_rows_kernel<kNT><<<(unsigned)srcs.size(), kNT, 0, s>>>(dv_src);
    bool t32 = false, t64 = false;  // entry widths present among the tasks' sources
    for (const KTask &t : tasks) (t.src.small ? t32 : t64) = true;
    {
        const size_t sm = contract_smem(maxN);
        if (t32) {
            CAC_TRY(smem_optin(ctx_, contract_kernel<kNT, uint32_t>));
            contract_kernel<kNT, uint32_t><<<(unsigned)tasks.size(), kNT, sm, s>>>(
                dv_task, dv_src, d_kout.as<uint32_t>(), d_err);
        }
        if (t64) {
            CAC_TRY(smem_optin(ctx_, contract_kernel<kNT, uint64_t>));
            contract_kernel<kNT, uint64_t><<<(unsigned)tasks.size(), kNT, sm, s>>>(
                dv_task, dv_src, d_kout.as<uint32_t>(), d_err);
        }
        CAC_CUDA_TRY(cudaGetLastError());
    }
    // the children's sizes: read back, or (planning ahead) taken to be their targets, which the
    // quotient kernels check against the contraction's own counts on the device
    std::vector<uint32_t> kk(tasks.size());
    const uint32_t *kact = nullptr;
    if (plan_ahead_) {
        for (size_t i = 0; i < tasks.size(); i++) kk[i] = tasks[i].target;
        kact = d_kout.as<uint32_t>();
    } else {
        CAC_CUDA_TRY(cudaMemcpyAsync(kk.data(), d_kout.p, tasks.size() * 4, cudaMemcpyDeviceToHost, s));
        CAC_CUDA_TRY(cudaStreamSynchronize(s));
    }

    // quotient matrices of this step, in one stream-ordered buffer: each child's matrix, then
    // (after all matrices) each child's row sums and 32-column block prefixes, which the quotient
    // kernels write for the next step's draws
    std::vector<uint64_t> out_off(2 * tasks.size(), 0);
    std::vector<uint32_t> kq(tasks.size(), 0);
    uint64_t out_bytes = 0;
    bool all_small = true;
    uint32_t kmax = 0;
    for (size_t i = 0; i < tasks.size(); i++) {
        const uint32_t k = kk[i] == kDropped ? 0 : kk[i];
        kq[i] = k;
        out_off[i] = out_bytes;
        out_bytes += ((uint64_t)k * ld_of(k) * (tasks[i].src.small ? 4 : 8) + 15) / 16 * 16;
        all_small = all_small && tasks[i].src.small;
        kmax = std::max(kmax, k);
    }
    for (size_t i = 0; i < tasks.size(); i++) {
        out_off[tasks.size() + i] = out_bytes;
        out_bytes += ((kq[i] + (uint64_t)kq[i] * ((kq[i] + 31) / 32)) * 8 + 15) / 16 * 16;
    }
    // Three quotient kernels, identical outputs: warp-per-row (8 or 4 warps, one k-entry row per
    // warp in shared memory; where three of its CTAs fit an SM: labels + rows within 80 KB), its
    // bulk-copy variant, and shared-row (8 warps on one output row). Which is fastest depends on
    // N, k and the task count, so the step autotunes: the first sizeable step of each
    // (power-of-two bucket of N, entry width) on this ctx times them on its own data and keeps the
    // fastest; smaller steps before that use the rule measured on GB300 (shared-row from N = 2000
    // on).
    const size_t stage_words = ((size_t)maxN + 3) & ~(size_t)3;  // N u32 labels, 16-byte rounded
    const size_t rs_bytes = all_small ? 4 : 8;
    const uint32_t qwarps = stage_words * 4 + 8 * rs_bytes * (size_t)kmax <= 80 * 1024   ? 8u
                            : stage_words * 4 + 4 * rs_bytes * (size_t)kmax <= 80 * 1024 ? 4u
                                                                                         : 0u;
    auto group_offsets = [&](uint32_t rows, std::vector<uint64_t> &gto) {
        gto.assign(tasks.size(), 0);
        uint64_t g = 0;
        for (size_t i = 0; i < tasks.size(); i++) {
            gto[i] = g;
            g += (kq[i] + rows - 1) / rows;
        }
        return g;
    };
    std::vector<uint64_t> gto_warp, gto_shared;
    const uint64_t groups_warp = qwarps ? group_offsets(qwarps * 4, gto_warp) : 0;
    const uint64_t groups_shared = group_offsets(kSharedRows, gto_shared);
    // the bulk-copy variant of the warp quotient: labels, then per warp two staged member rows
    // and its output row; 8 warps where two CTAs fit an SM, else 4 where one does
    const size_t row_words = (size_t)ld_of(maxN);
    const size_t bulk_per_warp = ((row_words * (all_small ? 4 : 8)) * 2 + (size_t)kmax * rs_bytes + 15) & ~(size_t)15;
    const size_t bulk_base = 128 + ((stage_words * 4 + 15) & ~(size_t)15);
    const uint32_t bwarps = bulk_base + 8 * bulk_per_warp <= 113 * 1024   ? 8u
                            : bulk_base + 4 * bulk_per_warp <= 226 * 1024 ? 4u
                                                                          : 0u;
    std::vector<uint64_t> gto_bulk;
    const uint64_t groups_bulk = bwarps ? group_offsets(bwarps * 4, gto_bulk) : 0;
    MatBuf *out = nullptr;
    if (groups_shared) {
        CAC_TRY(alloc(out_bytes, &out));
        // one descriptor copy for the output offsets, the children's sizes and the row groups
        CAC_TRY(post_st.begin(Staging::bytes_of(out_off) + Staging::bytes_of(kq) + Staging::bytes_of(gto_shared) +
                              Staging::bytes_of(gto_warp) + Staging::bytes_of(gto_bulk)));
        const uint64_t *dv_qoff = post_st.put(out_off);
        const uint32_t *dv_k = post_st.put(kq);
        const uint64_t *dv_gto_shared = post_st.put(gto_shared);
        const uint64_t *dv_gto_warp = post_st.put(gto_warp);
        const uint64_t *dv_gto_bulk = post_st.put(gto_bulk);
        CAC_TRY(post_st.flush());
        unsigned char *obase = static_cast<unsigned char *>(out->p);
        const uint32_t ntk = (uint32_t)tasks.size();
        auto launch_shared = [&]() -> int {
            const size_t ssm = stage_words * 4 + (((size_t)kmax * rs_bytes + 15) & ~(size_t)15) +
                               ((size_t)kmax / 32 + 1) * 8;
            std::vector<decltype(&quotient_shared_row_kernel<uint32_t, uint32_t>)> kerns;
            if (all_small) kerns.push_back(quotient_shared_row_kernel<uint32_t, uint32_t>);
            else {
                if (t32) kerns.push_back(quotient_shared_row_kernel<uint64_t, uint32_t>);
                if (t64) kerns.push_back(quotient_shared_row_kernel<uint64_t, uint64_t>);
            }
            for (auto kern : kerns) {
                CAC_TRY(smem_optin(ctx_, kern));
                kern<<<(unsigned)groups_shared, 256, ssm, s>>>(dv_task, dv_src, dv_k, dv_gto_shared, ntk, kSharedRows,
                                                               dv_qoff, obase, (uint32_t)stage_words, kmax, kact,
                                                               d_err);
            }
            CAC_CUDA_TRY(cudaGetLastError());
            return CAC_OK;
        };
        auto launch_warp = [&]() -> int {
            // shared rows are u32 only when every task's sums fit (all sources small)
            const size_t wsm = stage_words * 4 + (size_t)qwarps * kmax * rs_bytes;
            std::vector<decltype(&quotient_warp_kernel<uint32_t, uint32_t>)> kerns;
            if (all_small) kerns.push_back(quotient_warp_kernel<uint32_t, uint32_t>);
            else {
                if (t32) kerns.push_back(quotient_warp_kernel<uint64_t, uint32_t>);
                if (t64) kerns.push_back(quotient_warp_kernel<uint64_t, uint64_t>);
            }
            for (auto kern : kerns) {
                CAC_TRY(smem_optin(ctx_, kern));
                kern<<<(unsigned)groups_warp, qwarps * 32, wsm, s>>>(dv_task, dv_src, dv_k, dv_gto_warp, ntk,
                                                                     qwarps * 4, dv_qoff, obase,
                                                                     (uint32_t)stage_words, kmax, kact, d_err);
            }
            CAC_CUDA_TRY(cudaGetLastError());
            return CAC_OK;
        };
        auto launch_bulk = [&]() -> int {
            const size_t bsm = bulk_base + bwarps * bulk_per_warp;
            std::vector<decltype(&quotient_bulk_kernel<uint32_t, uint32_t>)> kerns;
            if (all_small) kerns.push_back(quotient_bulk_kernel<uint32_t, uint32_t>);
            else {
                if (t32) kerns.push_back(quotient_bulk_kernel<uint64_t, uint32_t>);
                if (t64) kerns.push_back(quotient_bulk_kernel<uint64_t, uint64_t>);
            }
            for (auto kern : kerns) {
                CAC_TRY(smem_optin(ctx_, kern));
                kern<<<(unsigned)groups_bulk, bwarps * 32, bsm, s>>>(dv_task, dv_src, dv_k, dv_gto_bulk, ntk,
                                                                     bwarps * 4, dv_qoff, obase,
                                                                     (uint32_t)stage_words, kmax,
                                                                     (uint32_t)row_words, d_err, kact);
            }
            CAC_CUDA_TRY(cudaGetLastError());
            return CAC_OK;
        };
        uint8_t &tuned = ctx_->quotient_forced ? ctx_->quotient_forced
                                               : ctx_->quotient_choice[quotient_bucket(maxN, all_small)];
        const bool sizeable = groups_shared >= (uint64_t)4 * ctx_->num_sms;  // enough work to time
        if (!qwarps && !bwarps) {
            CAC_TRY(launch_shared());
        } else if (tuned == kQuotientShared) {
            CAC_TRY(launch_shared());
        } else if (tuned == kQuotientWarp && qwarps) {
            CAC_TRY(launch_warp());
        } else if (tuned == kQuotientBulk && bwarps) {
            CAC_TRY(launch_bulk());
        } else if (!sizeable || tuned) {  // too small to time, already timed, or kQuotientRule forced
            CAC_TRY(maxN >= kSharedRowMinN || !qwarps ? launch_shared() : launch_warp());
        } else {
            // all write the same matrices, row sums and prefixes: time each on this step's data
            cudaEvent_t *ev = ctx_->ev;
            float t_warp = 1e30f, t_shared = 0, t_bulk = 1e30f;
            CAC_CUDA_TRY(cudaEventRecord(ev[4], s));
            if (qwarps) CAC_TRY(launch_warp());
            CAC_CUDA_TRY(cudaEventRecord(ev[5], s));
            if (bwarps) CAC_TRY(launch_bulk());
            CAC_CUDA_TRY(cudaEventRecord(ev[6], s));
            CAC_TRY(launch_shared());
            CAC_CUDA_TRY(cudaEventRecord(ev[7], s));
            CAC_CUDA_TRY(cudaEventSynchronize(ev[7]));
            if (qwarps) CAC_CUDA_TRY(cudaEventElapsedTime(&t_warp, ev[4], ev[5]));
            if (bwarps) CAC_CUDA_TRY(cudaEventElapsedTime(&t_bulk, ev[5], ev[6]));
            CAC_CUDA_TRY(cudaEventElapsedTime(&t_shared, ev[6], ev[7]));
            tuned = t_shared <= t_warp && t_shared <= t_bulk ? kQuotientShared
                    : t_bulk < t_warp                        ? kQuotientBulk
                                                             : kQuotientWarp;
        }
    }
    // the sources are read by everything enqueued above: their buffers may now be released
    for (MatBuf *b : consumed) release(b);
    for (size_t i = 0; i < tasks.size(); i++) {
        const KTask &t = tasks[i];
        outstanding[t.src.query]--;
        const uint32_t k = kq[i];
        if (k == 0) continue;  // dropped: the source had no edges, its cut 0 is recorded
        KNode nd = t.src;
        nd.h = t.h;
        nd.N = k;
        nd.is_root = 0;
        nd.mat = static_cast<unsigned char *>(out->p) + out_off[i];
        nd.pre = reinterpret_cast<uint64_t *>(static_cast<unsigned char *>(out->p) + out_off[tasks.size() + i]);
        nd.buf = out;
        out->refs++;
        outstanding[nd.query]++;
        if (k <= t.target) {
            nodes_.push_back(nd);
        } else {
            KTask c = t;
            c.src = nd;
            c.round += 1;
            carried_.push_back(c);
        }
    }
    if (out && out->refs == 0) {  // every child was dropped
        out->refs = 1;
        release(out);
    }
    return CAC_OK;
}

namespace {

// Admission of square_root queries: trial keys, per-trial cut slots, Stage 1 and Stage 2, root nodes.
struct QueryPlan {
    const cac_graph *g;
    uint32_t seed, ranks, per_rank;
    uint32_t t;
    uint64_t trials;
    uint64_t *cuts;       // device, one per trial
    uint32_t query;       // engine bookkeeping id
    uint32_t groups = 0;  // > 0: the high-concurrency group variant (trials = groups)
};

int admit_groups(cac_ctx *ctx, KsEngine &eng, const QueryPlan &q);

int admit_stage1(cac_ctx *ctx, KsEngine &eng, const std::vector<const QueryPlan *> &qs);
int admit_big(cac_ctx *ctx, KsEngine &eng, const QueryPlan &q);

// The sparse root of one square_root trial contracted to k vertices above the dense limit: the
// graph's edges relabelled by the trial's Stage 1 labels, sorted and merged on the device (the
// reference's WeightedIteratedSparseSampling::reduce, .cpp:26-234). The list's buffer carries
// the node's reference.
int sparse_root(cac_ctx *ctx, KsEngine &eng, const QueryPlan &q, uint64_t *cut, uint32_t k0, uint32_t idx,
                const uint32_t *lab, uint32_t k, SparseNode *out) {
    const cac_graph *g = q.g;
    const uint64_t cap = std::max<uint64_t>(g->m, 1);
    MatBuf *list = nullptr;
    CAC_TRY(eng.alloc(align_up(cap * 4) * 2 + align_up(cap * 8), &list));
    list->refs++;
    char *p = static_cast<char *>(list->p);
    uint32_t *oa = reinterpret_cast<uint32_t *>(p), *ob = reinterpret_cast<uint32_t *>(p + align_up(cap * 4));
    uint64_t *ow = reinterpret_cast<uint64_t *>(p + 2 * align_up(cap * 4));
    DevBuf &scr = scratch(ctx, kSlotSparse), &cnt = scratch(ctx, kSlotSparseCount);
    int st = scr.ensure(merge_edges_scratch(cap));
    if (st == CAC_OK) st = cnt.ensure(4);
    if (st == CAC_OK)
        st = merge_edges<uint32_t>(ctx, g->u, g->v, g->w, g->m, lab, k, oa, ob, ow, cnt.as<uint32_t>(), scr.p);
    uint32_t mm = 0;
    if (st == CAC_OK && (cudaMemcpyAsync(&mm, cnt.p, 4, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
                         cudaStreamSynchronize(ctx->stream) != cudaSuccess)) {
        set_error("square_root: reading the sparse root's edge count failed");
        st = CAC_ERR_CUDA;
    }
    if (st != CAC_OK) {
        eng.release(list);
        return st;
    }
    *out = SparseNode{cut, k0, idx, 1, k, k >= 2 ? mm : 0, oa, ob, ow, true, true,
                      g->total_weight < (1ull << 32) ? 1u : 0u, q.query, list};
    return CAC_OK;
}

int admit(cac_ctx *ctx, KsEngine &eng, const QueryPlan &q) {
    cudaStream_t s = ctx->stream;
    const cac_graph *g = q.g;
    const uint32_t n = g->n;
    const uint64_t m = g->m;
    const uint32_t small = g->total_weight < (1ull << 32) ? 1u : 0u;
    if (q.trials == 0) return CAC_OK;
    if (q.t >= n && !ks_is_dense(ctx, n, m)) {
        // No pre-contraction and a sparse graph: every trial starts from the input edge list. The
        // dense levels below the sparse ones hold about n^2 entries per level and trial, so the
        // trials run in groups that keep two such levels within the bound, each group to its end.
        const uint64_t per_trial = 2ull * n * n * (small ? 4 : 8);
        const uint64_t bound = ctx->budget ? ctx->budget / 2 : (32ull << 30);
        const uint64_t group = std::max<uint64_t>(1, std::min<uint64_t>(q.trials, bound / per_trial));
        for (uint64_t g0 = 0; g0 < q.trials; g0 += group) {
            std::vector<SparseNode> roots;
            for (uint64_t i = g0; i < std::min(q.trials, g0 + group); i++) {
                const uint32_t r = (uint32_t)(i / q.per_rank), idx = (uint32_t)(i % q.per_rank);
                roots.push_back(SparseNode{q.cuts + i, q.seed + r, idx, 1, n, m, g->u, g->v, g->w, false, true, small,
                                           q.query, nullptr});
            }
            CAC_TRY(sparse_phase(ctx, eng, std::move(roots)));
            if (g0 + group < q.trials)
                while (!eng.idle()) CAC_TRY(eng.step());
        }
        return CAC_OK;
    }
    if (q.t >= n) {
        // no pre-contraction: every trial starts from the same dense matrix, built once
        MatBuf *root = nullptr;
        const size_t bytes = (size_t)n * ld_of(n) * (small ? 4 : 8);
        CAC_TRY(eng.alloc(bytes, &root));
        CAC_CUDA_TRY(cudaMemsetAsync(root->p, 0, bytes, s));
        if (m) {
            DevBuf &d = scratch(ctx, kSlotDd);
            std::vector<DenseDesc> dd{DenseDesc{g->u, g->v, g->w, nullptr, root->p, m, n, small}};
            CAC_TRY(upload(ctx, d, dd));
            dim3 grid((unsigned)std::max<uint64_t>(1, std::min<uint64_t>((m + 255) / 256, (uint64_t)ctx->num_sms * 8)), 1);
            dense_build_kernel<<<grid, 256, 0, s>>>(d.as<DenseDesc>());
            CAC_CUDA_TRY(cudaGetLastError());
            CAC_CUDA_TRY(cudaStreamSynchronize(s));  // the descriptor buffer goes out of scope
        }
        root->refs++;  // held until every root node has been added
        for (uint64_t i = 0; i < q.trials; i++) {
            const uint32_t r = (uint32_t)(i / q.per_rank), idx = (uint32_t)(i % q.per_rank);
            eng.add(KNode{q.cuts + i, q.seed + r, idx, 1, n, 1, small, q.query, root->p, root});
        }
        eng.release(root);
        return CAC_OK;
    }
    // Stage 1: the global-memory rounds of shrink_big.cu above 16384 vertices, else the
    // shared-memory kernel, batched with other queries' trials where the caller has several
    if (n > kMaxSmemVertices) return admit_big(ctx, eng, q);
    std::vector<const QueryPlan *> one{&q};
    return admit_stage1(ctx, eng, one);
}

// Stage 1 and Stage 2 of every trial of the given queries (t < n <= 16384), the trials of all of
// them together: one Stage 1 launch, one read-back of the contracted sizes and one dense build
// per chunk, whose scratch stays within 4 GB. Admitting the queries of a batch one by one costs a
// launch and two host synchronisations per query.
int admit_stage1(cac_ctx *ctx, KsEngine &eng, const std::vector<const QueryPlan *> &qs) {
    cudaStream_t s = ctx->stream;
    struct Item {
        const QueryPlan *q;
        uint64_t i;
    };
    std::vector<Item> items;
    for (const QueryPlan *q : qs)
        for (uint64_t i = 0; i < q->trials; i++) items.push_back({q, i});
    DevBuf &d_pre = scratch(ctx, kSlotPre), &d_lab = scratch(ctx, kSlotLab), &d_k = scratch(ctx, kSlotK),
           &d_sd = scratch(ctx, kSlotSd), &d_dd = scratch(ctx, kSlotDd);
    CAC_TRY(smem_optin(ctx, iss_shrink_kernel<kNT>));
    size_t c0 = 0;
    while (c0 < items.size()) {
        // a chunk: at most 65535 trials and 4 GB of prefix + label scratch
        size_t c1 = c0;
        uint64_t pre_words = 0, lab_words = 0;
        uint32_t nmax = 1;
        uint64_t mmax = 1;
        while (c1 < items.size() && c1 - c0 < 65535) {
            const cac_graph *g = items[c1].q->g;
            const uint64_t pw = std::max<uint64_t>(g->m, 1), lw = g->n;
            if (c1 > c0 && (pre_words + pw) * 8 + (lab_words + lw) * 4 > (4ull << 30)) break;
            pre_words += pw;
            lab_words += lw;
            nmax = std::max(nmax, g->n);
            mmax = std::max(mmax, g->m);
            c1++;
        }
        const uint32_t B = (uint32_t)(c1 - c0);
        CAC_TRY(d_pre.ensure(pre_words * 8));
        CAC_TRY(d_lab.ensure(lab_words * 4));
        CAC_TRY(d_k.ensure((size_t)B * 4));
        std::vector<ShrinkDesc> sd(B);
        uint64_t po = 0, lo = 0;
        for (uint32_t b = 0; b < B; b++) {
            const QueryPlan &q = *items[c0 + b].q;
            const uint64_t i = items[c0 + b].i;
            ShrinkDesc &D = sd[b];
            D.U = q.g->u;
            D.V = q.g->v;
            D.W = q.g->w;
            D.m = q.g->m;
            D.pre = d_pre.as<uint64_t>() + po;
            D.lab = d_lab.as<uint32_t>() + lo;
            D.k_out = d_k.as<uint32_t>() + b;
            D.n = q.g->n;
            D.target = q.t;
            D.k0 = q.seed + (uint32_t)(i / q.per_rank);
            D.idx = (uint32_t)(i % q.per_rank);
            po += std::max<uint64_t>(q.g->m, 1);
            lo += q.g->n;
        }
        const size_t sm = kBatch * sizeof(uint2) + kCoarse * sizeof(uint64_t) + (size_t)nmax * 4;
        CAC_TRY(upload(ctx, d_sd, sd));
        // fewer trials than SMs: one trial per SM either way, so each trial gets 1024 threads
        if (B < (uint32_t)ctx->num_sms) {
            CAC_TRY(smem_optin(ctx, iss_shrink_kernel<2 * kNT>));
            iss_shrink_kernel<2 * kNT><<<B, 2 * kNT, sm, s>>>(d_sd.as<ShrinkDesc>());
        } else {
            iss_shrink_kernel<kNT><<<B, kNT, sm, s>>>(d_sd.as<ShrinkDesc>());
        }
        CAC_CUDA_TRY(cudaGetLastError());
        // the contracted sizes: read back, or (planning ahead, no sparse root in the chunk) taken to
        // be the targets, which the dense build checks against Stage 1's counts on the device
        bool sparse_roots = false;
        for (uint32_t b = 0; b < B; b++) sparse_roots = sparse_roots || items[c0 + b].q->t > ctx->dense_limit;
        const bool planned = eng.plan_ahead() && !sparse_roots;
        std::vector<uint32_t> kdim(B);
        if (planned) {
            for (uint32_t b = 0; b < B; b++) kdim[b] = items[c0 + b].q->t;
        } else {
            CAC_CUDA_TRY(cudaMemcpyAsync(kdim.data(), d_k.p, (size_t)B * 4, cudaMemcpyDeviceToHost, s));
            CAC_CUDA_TRY(cudaStreamSynchronize(s));
        }
        // trials contracted to more than the dense limit: sparse roots (sorted, merged edge lists)
        std::vector<SparseNode> sparse;
        for (uint32_t b = 0; b < B; b++) {
            const QueryPlan &q = *items[c0 + b].q;
            if (q.t <= ctx->dense_limit) continue;
            SparseNode nd;
            CAC_TRY(sparse_root(ctx, eng, q, q.cuts + items[c0 + b].i, sd[b].k0, sd[b].idx, sd[b].lab, kdim[b], &nd));
            sparse.push_back(nd);
            kdim[b] = 0;  // no dense matrix
        }
        uint64_t bytes = 0;
        for (uint32_t b = 0; b < B; b++) {
            const uint64_t esize = items[c0 + b].q->g->total_weight < (1ull << 32) ? 4 : 8;
            bytes += ((uint64_t)kdim[b] * ld_of(kdim[b]) * esize + 15) / 16 * 16;
        }
        MatBuf *roots = nullptr;
        CAC_TRY(eng.alloc(std::max<uint64_t>(bytes, 16), &roots));
        CAC_CUDA_TRY(cudaMemsetAsync(roots->p, 0, bytes, s));
        std::vector<DenseDesc> dd(B);
        uint64_t off = 0;
        for (uint32_t b = 0; b < B; b++) {
            const cac_graph *g = items[c0 + b].q->g;
            const uint32_t small = g->total_weight < (1ull << 32) ? 1u : 0u;
            // no scatter for a trial without a matrix (its labels would index past the buffer)
            dd[b] = DenseDesc{g->u, g->v, g->w, sd[b].lab, static_cast<unsigned char *>(roots->p) + off,
                              kdim[b] >= 2 ? g->m : 0, kdim[b], small};
            if (planned) {
                dd[b].k_act = sd[b].k_out;
                dd[b].err = eng.err_word();
            }
            off += ((uint64_t)kdim[b] * ld_of(kdim[b]) * (small ? 4 : 8) + 15) / 16 * 16;
        }
        CAC_TRY(upload(ctx, d_dd, dd));
        dim3 grid((unsigned)std::max<uint64_t>(
                      1, std::min<uint64_t>((mmax + 255) / 256, std::max<uint64_t>(1, (uint64_t)ctx->num_sms * 8 / B))),
                  B);
        dense_build_kernel<<<grid, 256, 0, s>>>(d_dd.as<DenseDesc>());
        CAC_CUDA_TRY(cudaGetLastError());
        roots->refs++;
        for (uint32_t b = 0; b < B; b++) {
            const QueryPlan &q = *items[c0 + b].q;
            const uint64_t i = items[c0 + b].i;
            if (q.t > ctx->dense_limit) continue;  // a sparse root
            if (kdim[b] < 2) {
                // a single vertex left, or only isolated vertices: no cut edge
                fill_u64<<<1, 32, 0, s>>>(q.cuts + i, 1, 0);
                continue;
            }
            eng.add(KNode{q.cuts + i, sd[b].k0, sd[b].idx, 1, kdim[b], 1, dd[b].small, q.query, dd[b].mat, roots});
        }
        eng.release(roots);
        // the scratch is refilled from the host for the next chunk (later kernels on the stream
        // are ordered after these, so the last chunk needs no wait)
        if (c1 < items.size()) CAC_CUDA_TRY(cudaStreamSynchronize(s));
        if (!sparse.empty()) CAC_TRY(sparse_phase(ctx, eng, std::move(sparse)));
        c0 = c1;
    }
    return CAC_OK;
}

// Stage 1 of a query above 16384 vertices: the global-memory rounds of shrink_big.cu, in chunks
// of trials whose scratch stays within 4 GB.
int admit_big(cac_ctx *ctx, KsEngine &eng, const QueryPlan &q) {
    cudaStream_t s = ctx->stream;
    const cac_graph *g = q.g;
    const uint32_t n = g->n;
    const uint64_t m = g->m;
    const uint32_t small = g->total_weight < (1ull << 32) ? 1u : 0u;
    const uint64_t per_trial = shrink_big_scratch(n, m, 1) + 4ull * n;
    const uint64_t chunk = std::max<uint64_t>(1, std::min<uint64_t>({q.trials, (4ull << 30) / per_trial, (uint64_t)65535}));
    DevBuf &d_pre = scratch(ctx, kSlotPre), &d_lab = scratch(ctx, kSlotLab), &d_k = scratch(ctx, kSlotK),
           &d_dd = scratch(ctx, kSlotDd);
    for (uint64_t c0 = 0; c0 < q.trials; c0 += chunk) {
        const uint32_t B = (uint32_t)std::min<uint64_t>(chunk, q.trials - c0);
        CAC_TRY(d_pre.ensure(shrink_big_scratch(n, m, B)));
        CAC_TRY(d_lab.ensure((size_t)B * n * 4));
        CAC_TRY(d_k.ensure((size_t)B * 4));
        std::vector<uint32_t> k0(B), idx(B);
        for (uint32_t b = 0; b < B; b++) {
            const uint64_t i = c0 + b;
            k0[b] = q.seed + (uint32_t)(i / q.per_rank);
            idx[b] = (uint32_t)(i % q.per_rank);
        }
        CAC_TRY(shrink_big(ctx, g, q.t, B, k0.data(), idx.data(), d_lab.as<uint32_t>(), d_k.as<uint32_t>(), d_pre.p));
        std::vector<uint32_t> kdim(B);
        CAC_CUDA_TRY(cudaMemcpyAsync(kdim.data(), d_k.p, (size_t)B * 4, cudaMemcpyDeviceToHost, s));
        CAC_CUDA_TRY(cudaStreamSynchronize(s));
        // trials contracted above the dense limit become sparse roots; otherwise more than 16384
        // vertices are left only when Stage 1 stopped with no edge between them (a disconnected
        // graph): every vertex is isolated and the trial's cut is exactly 0
        std::vector<SparseNode> sparse;
        for (uint32_t b = 0; b < B; b++) {
            if (q.t > ctx->dense_limit) {
                SparseNode nd;
                CAC_TRY(sparse_root(ctx, eng, q, q.cuts + c0 + b, k0[b], idx[b], d_lab.as<uint32_t>() + (size_t)b * n,
                                    kdim[b], &nd));
                sparse.push_back(nd);
                kdim[b] = 0;
            } else if (kdim[b] > kMaxSmemVertices) {
                kdim[b] = 0;
            }
        }
        const uint64_t esize = small ? 4 : 8;
        uint64_t bytes = 0;
        for (uint32_t b = 0; b < B; b++) bytes += ((uint64_t)kdim[b] * ld_of(kdim[b]) * esize + 15) / 16 * 16;
        MatBuf *roots = nullptr;
        CAC_TRY(eng.alloc(std::max<uint64_t>(bytes, 16), &roots));
        CAC_CUDA_TRY(cudaMemsetAsync(roots->p, 0, bytes, s));
        std::vector<DenseDesc> dd(B);
        uint64_t off = 0;
        for (uint32_t b = 0; b < B; b++) {
            // no scatter for a trial without a matrix (its labels would index past the buffer)
            dd[b] = DenseDesc{g->u, g->v, g->w, d_lab.as<uint32_t>() + (size_t)b * n,
                              static_cast<unsigned char *>(roots->p) + off, kdim[b] >= 2 ? m : 0, kdim[b], small};
            off += ((uint64_t)kdim[b] * ld_of(kdim[b]) * esize + 15) / 16 * 16;
        }
        CAC_TRY(upload(ctx, d_dd, dd));
        if (m) {
            dim3 grid((unsigned)std::max<uint64_t>(1, std::min<uint64_t>((m + 255) / 256, std::max<uint64_t>(1, (uint64_t)ctx->num_sms * 8 / B))), B);
            dense_build_kernel<<<grid, 256, 0, s>>>(d_dd.as<DenseDesc>());
            CAC_CUDA_TRY(cudaGetLastError());
        }
        roots->refs++;
        for (uint32_t b = 0; b < B; b++) {
            const uint64_t i = c0 + b;
            if (q.t > ctx->dense_limit) continue;  // a sparse root
            if (kdim[b] < 2) {
                fill_u64<<<1, 32, 0, s>>>(q.cuts + i, 1, 0);
                continue;
            }
            eng.add(KNode{q.cuts + i, k0[b], idx[b], 1, kdim[b], 1, small, q.query, dd[b].mat, roots});
        }
        eng.release(roots);
        if (c0 + chunk < q.trials) CAC_CUDA_TRY(cudaStreamSynchronize(s));  // the scratch is reused by the next chunk
        if (!sparse.empty()) CAC_TRY(sparse_phase(ctx, eng, std::move(sparse)));
    }
    return CAC_OK;
}

// The high-concurrency group variant (SquareRootCut::participateInGroup, SquareRootCut.cpp:188-298):
// group trial g runs WeightedIteratedSparseSampling::shrink (.cpp:4-24) as Stage 1 rounds of a
// fixed floor(n^1.05) weighted draws (edgesToSamplePerProcessor, .hpp:66-67) with key
// (seed + g, 0, 1, 0), builds the contracted graph (reduce, .cpp:26-234: dense, or a sorted and
// merged sparse root above the dense limit), and, as parallel_cut(.., 2, ..) runs two recursive
// contractions of it (recursive_contract.cpp:45-83), starts two Karger-Stein recursions from that
// root with keys (seed + g, 0 | 1, 1 + h, 0). All groups' Stage 1 runs in one grid per chunk
// (shrink_big.cu with a fixed draw count per round).
int admit_groups(cac_ctx *ctx, KsEngine &eng, const QueryPlan &q) {
    cudaStream_t s = ctx->stream;
    const cac_graph *g = q.g;
    const uint32_t n = g->n;
    const uint64_t m = g->m;
    const uint32_t small = g->total_weight < (1ull << 32) ? 1u : 0u;
    const bool stage1 = q.t < n;
    const uint32_t dpr = group_draws(n);
    const uint64_t tt = std::min<uint64_t>(q.t, n);
    const uint64_t per_group = (stage1 ? shrink_task_scratch(n, m, dpr) : 0) + 4ull * n +
                               (q.t > ctx->dense_limit ? 16ull * m : tt * ld_of((uint32_t)tt) * (small ? 4 : 8));
    const uint64_t chunk = std::max<uint64_t>(1, std::min<uint64_t>({q.trials, (4ull << 30) / per_group, (uint64_t)65535}));
    DevBuf &d_pre = scratch(ctx, kSlotPre), &d_lab = scratch(ctx, kSlotLab), &d_k = scratch(ctx, kSlotK),
           &d_dd = scratch(ctx, kSlotDd);
    for (uint64_t c0 = 0; c0 < q.trials; c0 += chunk) {
        const uint32_t B = (uint32_t)std::min<uint64_t>(chunk, q.trials - c0);
        std::vector<uint32_t> kdim(B, n);
        if (stage1) {
            std::vector<ShrinkTask> tasks(B);
            CAC_TRY(d_lab.ensure((size_t)B * n * 4));
            CAC_TRY(d_k.ensure((size_t)B * 4));
            for (uint32_t b = 0; b < B; b++)
                tasks[b] = ShrinkTask{g->u, g->v, g->w, false, m, n, q.t, q.seed + (uint32_t)(c0 + b), 0, 1,
                                      d_lab.as<uint32_t>() + (size_t)b * n, d_k.as<uint32_t>() + b, dpr};
            CAC_TRY(d_pre.ensure(shrink_tasks_scratch(tasks)));
            CAC_TRY(shrink_tasks(ctx, tasks, d_pre.p));
            CAC_CUDA_TRY(cudaMemcpyAsync(kdim.data(), d_k.p, (size_t)B * 4, cudaMemcpyDeviceToHost, s));
            CAC_CUDA_TRY(cudaStreamSynchronize(s));
        }
        auto lab_of = [&](uint32_t b) -> const uint32_t * {
            return stage1 ? d_lab.as<uint32_t>() + (size_t)b * n : nullptr;
        };
        if (q.t > ctx->dense_limit) {
            // sparse roots: the merged contracted graph, shared by the group's two recursions
            std::vector<SparseNode> sparse;
            for (uint32_t b = 0; b < B; b++) {
                SparseNode nd;
                CAC_TRY(sparse_root(ctx, eng, q, q.cuts + c0 + b, q.seed + (uint32_t)(c0 + b), 0, lab_of(b), kdim[b],
                                    &nd));
                sparse.push_back(nd);
                nd.idx = 1;
                if (nd.buf) nd.buf->refs++;
                sparse.push_back(nd);
            }
            CAC_TRY(sparse_phase(ctx, eng, std::move(sparse)));
            continue;
        }
        // dense roots (more than 16384 vertices left only when Stage 1 found no edge between
        // them: a disconnected graph, cut 0)
        for (uint32_t b = 0; b < B; b++)
            if (kdim[b] > kMaxSmemVertices) kdim[b] = 0;
        const uint64_t esize = small ? 4 : 8;
        uint64_t bytes = 0;
        for (uint32_t b = 0; b < B; b++) bytes += ((uint64_t)kdim[b] * ld_of(kdim[b]) * esize + 15) / 16 * 16;
        MatBuf *roots = nullptr;
        CAC_TRY(eng.alloc(std::max<uint64_t>(bytes, 16), &roots));
        CAC_CUDA_TRY(cudaMemsetAsync(roots->p, 0, bytes, s));
        std::vector<DenseDesc> dd(B);
        uint64_t off = 0;
        for (uint32_t b = 0; b < B; b++) {
            dd[b] = DenseDesc{g->u, g->v, g->w, lab_of(b), static_cast<unsigned char *>(roots->p) + off,
                              kdim[b] >= 2 ? m : 0, kdim[b], small};
            off += ((uint64_t)kdim[b] * ld_of(kdim[b]) * esize + 15) / 16 * 16;
        }
        CAC_TRY(upload(ctx, d_dd, dd));
        if (m) {
            dim3 grid((unsigned)std::max<uint64_t>(
                          1, std::min<uint64_t>((m + 255) / 256, std::max<uint64_t>(1, (uint64_t)ctx->num_sms * 8 / B))),
                      B);
            dense_build_kernel<<<grid, 256, 0, s>>>(d_dd.as<DenseDesc>());
            CAC_CUDA_TRY(cudaGetLastError());
        }
        roots->refs++;
        for (uint32_t b = 0; b < B; b++) {
            const uint64_t i = c0 + b;
            if (kdim[b] < 2) {
                fill_u64<<<1, 32, 0, s>>>(q.cuts + i, 1, 0);
                continue;
            }
            for (uint32_t j = 0; j < 2; j++)
                eng.add(KNode{q.cuts + i, q.seed + (uint32_t)i, j, 1, kdim[b], 1, small, q.query, dd[b].mat, roots});
        }
        eng.release(roots);
        if (c0 + chunk < q.trials) CAC_CUDA_TRY(cudaStreamSynchronize(s));  // the scratch is reused
    }
    return CAC_OK;
}

// Admission of several queries: those with Stage 1 in shared memory go through admit_stage1
// together, the others one by one.
int admit_many(cac_ctx *ctx, KsEngine &eng, const std::vector<const QueryPlan *> &qs) {
    std::vector<const QueryPlan *> batched;
    for (const QueryPlan *q : qs) {
        if (q->trials == 0) continue;
        if (q->groups) CAC_TRY(admit_groups(ctx, eng, *q));
        else if (q->t < q->g->n && q->g->n <= kMaxSmemVertices) batched.push_back(q);
        else CAC_TRY(admit(ctx, eng, *q));
    }
    return batched.empty() ? CAC_OK : admit_stage1(ctx, eng, batched);
}

int check_graph(const cac_graph *g, uint32_t t_override) {
    if (g->total_weight >= (1ull << 55)) {
        set_error("total edge weight >= 2^55 is not supported by the Stoer-Wagner leaf kernel");
        return CAC_ERR_UNSUPPORTED;
    }
    (void)t_override;  // contracted sizes above the dense limit run as sparse roots
    return CAC_OK;
}

}  // namespace

int mincut_admit_queries(cac_ctx *ctx, KsEngine &eng, const std::vector<MincutQuery> &qs,
                         const std::vector<uint32_t> &ids, std::vector<int> &status, std::vector<std::string> &msgs) {
    status.assign(qs.size(), CAC_OK);
    msgs.assign(qs.size(), std::string());
    std::vector<QueryPlan> plans;
    plans.reserve(qs.size());
    std::vector<size_t> which;
    for (size_t i = 0; i < qs.size(); i++) {
        const MincutQuery &q = qs[i];
        const int st = check_graph(q.g, q.t);
        if (st != CAC_OK) {
            status[i] = st;
            msgs[i] = cac_last_error();
            continue;
        }
        plans.push_back(QueryPlan{q.g, q.seed, q.ranks, q.per_rank, q.t ? q.t : intermediate_size(q.g->n, q.g->m),
                                  q.groups ? (uint64_t)q.groups : (uint64_t)q.ranks * q.per_rank, q.d_cuts, ids[i],
                                  q.groups});
        which.push_back(i);
        const QueryPlan &p = plans.back();
        if (p.trials)
            fill_u64<<<(unsigned)std::max<uint64_t>(1, std::min<uint64_t>((p.trials + 255) / 256, 4096)), 256, 0,
                       ctx->stream>>>(p.cuts, p.trials, kU64Max);
    }
    if (cudaGetLastError() != cudaSuccess) {
        set_error("mincut_admit_queries: filling the trial slots failed");
        for (size_t i : which) {
            status[i] = CAC_ERR_CUDA;
            msgs[i] = cac_last_error();
        }
        return CAC_ERR_CUDA;
    }
    std::vector<const QueryPlan *> ptrs;
    for (const QueryPlan &p : plans) ptrs.push_back(&p);
    const int st = admit_many(ctx, eng, ptrs);
    if (st != CAC_OK)
        for (size_t i : which) {
            status[i] = st;
            msgs[i] = cac_last_error();
        }
    return st;
}

namespace {

// One run of the queries through one engine; *redo is set when a run that planned ahead met a child
// off its target (its cuts are then not valid, and the caller runs the queries again without).
int run_queries(cac_ctx *ctx, std::vector<MincutQuery> &queries, float *device_ms, bool plan_ahead, bool *redo) {
    cudaStream_t s = ctx->stream;
    CAC_CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
    KsEngine eng(ctx);
    eng.set_plan_ahead(plan_ahead);
    CAC_TRY(eng.init_err());
    std::vector<QueryPlan> plans(queries.size());
    for (size_t i = 0; i < queries.size(); i++) {
        MincutQuery &q = queries[i];
        QueryPlan &p = plans[i];
        p.g = q.g;
        p.seed = q.seed;
        p.ranks = q.ranks;
        p.per_rank = q.per_rank;
        p.t = q.t ? q.t : intermediate_size(q.g->n, q.g->m);
        p.trials = q.groups ? (uint64_t)q.groups : (uint64_t)q.ranks * q.per_rank;
        p.groups = q.groups;
        p.cuts = q.d_cuts;
        p.query = (uint32_t)i;
        if (p.trials)
            fill_u64<<<(unsigned)std::max<uint64_t>(1, std::min<uint64_t>((p.trials + 255) / 256, 4096)), 256, 0, s>>>(
                p.cuts, p.trials, kU64Max);
    }
    // admission by memory: a query is admitted when the engine's buffers leave room for its
    // estimated footprint (roots and two more levels of matrices); otherwise the engine steps first
    const uint64_t budget = ctx->budget ? ctx->budget / 2 : (48ull << 30);
    size_t next = 0;
    while (next < plans.size() || !eng.idle()) {
        // the queries that fit are admitted together (one Stage 1 launch for all of them)
        std::vector<const QueryPlan *> wave;
        uint64_t wave_est = 0;
        while (next < plans.size()) {
            const QueryPlan &p = plans[next];
            const uint64_t t = std::min<uint64_t>(p.t, p.g->n);
            const uint64_t est = (p.t < p.g->n ? p.trials : 1) * t * t * 8 * 3;
            if ((!eng.idle() || !wave.empty()) && ctx->held + wave_est + est > budget) break;
            wave.push_back(&p);
            wave_est += est;
            next++;
        }
        if (!wave.empty()) CAC_TRY(admit_many(ctx, eng, wave));
        if (!eng.idle()) CAC_TRY(eng.step());
    }
    uint32_t err = 0;
    CAC_TRY(eng.read_err(&err));
    CAC_CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
    CAC_CUDA_TRY(cudaStreamSynchronize(s));
    if (device_ms) CAC_CUDA_TRY(cudaEventElapsedTime(device_ms, ctx->ev[0], ctx->ev[1]));
    if (plan_ahead && (err & kErrPlan)) {
        *redo = true;
        return CAC_OK;
    }
    if (err) return engine_error(err);
    return CAC_OK;
}

}  // namespace

// Runs the queries planning ahead (no read-back of children's sizes between levels) when the ctx
// allows it; the rare run in which a child stops off its target is run again level by level. Both
// give the same cuts: every draw is addressed by its trial, node and round, not by the schedule.
int mincut_run_queries(cac_ctx *ctx, std::vector<MincutQuery> &queries, float *device_ms) {
    for (const MincutQuery &q : queries) CAC_TRY(check_graph(q.g, q.t));
    bool redo = false;
    float ms = 0;
    CAC_TRY(run_queries(ctx, queries, &ms, ctx->plan_ahead, &redo));
    if (redo) {
        float ms2 = 0;
        CAC_TRY(run_queries(ctx, queries, &ms2, false, &redo));
        ms += ms2;
        ctx->plan_redos++;
    }
    if (device_ms) *device_ms = ms;
    return CAC_OK;
}

int mincut_trials(cac_ctx *ctx, const cac_graph *g, uint32_t seed, uint32_t ranks, uint32_t per_rank,
                  uint64_t *d_cuts, float *device_ms) {
    std::vector<MincutQuery> q{MincutQuery{g, seed, ranks, per_rank, d_cuts}};
    return mincut_run_queries(ctx, q, device_ms);
}

// A dense host matrix for the device: checks the weight bound and, when the total weight is below
// 2^32 (and so every entry), narrows it to the u32 node storage.
int host_matrix(uint32_t n, const uint64_t *mat_host, uint32_t *small, std::vector<unsigned char> &dev) {
    uint64_t total = 0, top = 0;
    for (uint64_t i = 0; i < (uint64_t)n * n; i++) {
        total += mat_host[i];
        top = std::max(top, mat_host[i]);
    }
    if (total / 2 >= (1ull << 55)) {
        set_error("total edge weight >= 2^55 is not supported");
        return CAC_ERR_UNSUPPORTED;
    }
    *small = (total / 2 < (1ull << 32) && top < (1ull << 32)) ? 1u : 0u;
    // the device layout: rows padded to ld_of(n) entries of 4 or 8 bytes
    const uint64_t ld = ld_of(n), es = *small ? 4 : 8;
    dev.assign(n * ld * es, 0);
    for (uint64_t i = 0; i < n; i++)
        for (uint64_t j = 0; j < n; j++) {
            const uint64_t x = mat_host[i * n + j];
            if (*small) reinterpret_cast<uint32_t *>(dev.data())[i * ld + j] = (uint32_t)x;
            else reinterpret_cast<uint64_t *>(dev.data())[i * ld + j] = x;
        }
    return CAC_OK;
}

int ks_dense_one(cac_ctx *ctx, uint32_t n, const uint64_t *mat_host, uint32_t seed, uint32_t rank, uint32_t trial,
                 uint64_t *cut) {
    if (n > kMaxSmemVertices) {
        set_error("dense Karger-Stein supports at most 16384 vertices");
        return CAC_ERR_UNSUPPORTED;
    }
    std::vector<unsigned char> dev;
    uint32_t small = 0;
    CAC_TRY(host_matrix(n, mat_host, &small, dev));
    cudaStream_t s = ctx->stream;
    DevBuf &d_cut = scratch(ctx, kSlotProbe0);
    CAC_TRY(d_cut.ensure(8));
    {
        KsEngine eng(ctx);
        CAC_TRY(eng.init_err());
        MatBuf *root = nullptr;
        CAC_TRY(eng.alloc(dev.size(), &root));
        CAC_CUDA_TRY(cudaMemcpyAsync(root->p, dev.data(), dev.size(), cudaMemcpyHostToDevice, s));
        CAC_CUDA_TRY(cudaStreamSynchronize(s));  // `dev` is pageable and goes out of scope
        fill_u64<<<1, 32, 0, s>>>(d_cut.as<uint64_t>(), 1, kU64Max);
        eng.add(KNode{d_cut.as<uint64_t>(), seed + rank, trial, 1, n, 1, small, 0, root->p, root});
        while (!eng.idle()) CAC_TRY(eng.step());
        uint32_t err = 0;
        CAC_TRY(eng.read_err(&err));
        if (err) {
            return engine_error(err);
        }
    }
    CAC_CUDA_TRY(cudaMemcpyAsync(cut, d_cut.p, 8, cudaMemcpyDeviceToHost, s));
    CAC_CUDA_TRY(cudaStreamSynchronize(s));
    return CAC_OK;
}

int exact_small(cac_ctx *ctx, uint32_t n, const uint64_t *mat_host, uint64_t *cut) {
    std::vector<unsigned char> dev;
    uint32_t small = 0;
    CAC_TRY(host_matrix(n, mat_host, &small, dev));
    cudaStream_t s = ctx->stream;
    DevBuf &buf = scratch(ctx, kSlotProbe0), &d_cuts = scratch(ctx, kSlotProbe1), &d_leaf = scratch(ctx, kSlotProbe2);
    CAC_TRY(buf.ensure(dev.size()));
    CAC_TRY(d_cuts.ensure(8));
    CAC_CUDA_TRY(cudaMemcpyAsync(buf.p, dev.data(), dev.size(), cudaMemcpyHostToDevice, s));
    fill_u64<<<1, 32, 0, s>>>(d_cuts.as<uint64_t>(), 1, kU64Max);
    std::vector<LeafDesc> leaves{LeafDesc{buf.p, d_cuts.as<uint64_t>(), nullptr, n, small}};
    CAC_TRY(upload(ctx, d_leaf, leaves));
    if (small) {
        const size_t sm = leaf_smem(n, true);
        CAC_TRY(smem_optin(ctx, sw_leaf_kernel<uint32_t>));
        sw_leaf_kernel<uint32_t><<<1, kLeafThreads, sm, s>>>(d_leaf.as<LeafDesc>());
    } else {
        const size_t sm = leaf_smem(n, false);
        CAC_TRY(smem_optin(ctx, sw_leaf_kernel<uint64_t>));
        sw_leaf_kernel<uint64_t><<<1, kLeafThreads, sm, s>>>(d_leaf.as<LeafDesc>());
    }
    CAC_CUDA_TRY(cudaGetLastError());
    CAC_CUDA_TRY(cudaMemcpyAsync(cut, d_cuts.p, 8, cudaMemcpyDeviceToHost, s));
    CAC_CUDA_TRY(cudaStreamSynchronize(s));
    return CAC_OK;
}

}  // namespace cac
