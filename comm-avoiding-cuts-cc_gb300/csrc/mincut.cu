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
//              quotient_kernel   one CTA per output row: member rows summed by column label in
//                                shared memory (u64 shared atomics), one coalesced row store
//              sw_leaf_kernel    one warp per leaf (n <= 128): Stoer-Wagner maximum-adjacency
//                                phases on the matrix held in shared memory; atomicMin into the
//                                trial's cut
// The random stream of every draw is addressed by (seed + r, i, tag, 0) and (round, draw index),
// tag 1 for Stage 1 and 1 + h for the Karger-Stein child with heap index h, so a CPU replay of
// the same trial reproduces it bit for bit (oracle/mincut.c).
#include "cac_internal.h"
#include "sitmo.cuh"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace cac {
namespace {

constexpr uint32_t kMaxSmemVertices = 16384;  // union-find of a contraction held in shared memory
constexpr int kBatch = 1024;                  // draws gathered before the ordered contraction
constexpr int kNT = 512;                      // threads of the per-trial / per-task CTAs
constexpr int kQT = 256;                      // threads of the quotient CTAs
constexpr uint32_t kDropped = 0xFFFFFFFFu;    // task whose source matrix has no edges left
constexpr uint64_t kU64Max = 0xFFFFFFFFFFFFFFFFull;

struct TrialKey {
    uint32_t k0;   // seed + virtual rank
    uint32_t idx;  // trial index within the rank
};

struct SrcDesc {
    const uint64_t *mat;  // N x N row-major
    uint64_t *rowpre;     // N: inclusive prefix of row sums
    uint64_t *blk;        // N x nb: per row, inclusive prefix of 32-column block sums
    uint32_t N, nb;
    uint32_t trial;
    uint32_t is_root;     // root matrices also deliver the minimum weighted degree bound
};

struct TaskDesc {
    uint64_t tag;         // stream key word 2 (1 + heap index)
    uint32_t src;         // index into the SrcDesc array
    uint32_t target;
    uint32_t round;
    uint32_t trial;       // trial slot (index into cuts)
    uint32_t k0, idx;     // stream key words 0, 1
    uint32_t *lab;        // N labels (output)
    uint32_t *memb_off;   // k + 1 offsets (output)
    uint32_t *members;    // N vertices grouped by label (output)
};

struct LeafDesc {
    const uint64_t *mat;
    uint32_t N;
    uint32_t trial;
};

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

template <int NT>
__global__ void __launch_bounds__(NT) iss_shrink_kernel(uint32_t n, uint64_t m, const uint32_t *__restrict__ U,
                                                         const uint32_t *__restrict__ V,
                                                         const uint32_t *__restrict__ Wt, uint32_t target,
                                                         const TrialKey *__restrict__ keys,
                                                         uint64_t *__restrict__ pre_all, uint32_t *__restrict__ lab_all,
                                                         uint32_t *__restrict__ k_out) {
    extern __shared__ __align__(16) unsigned char dsm[];
    uint2 *sb = reinterpret_cast<uint2 *>(dsm);
    uint32_t *par = reinterpret_cast<uint32_t *>(dsm + kBatch * sizeof(uint2));
    __shared__ uint32_t s_count;
    const uint32_t t = blockIdx.x;
    const TrialKey key = keys[t];
    uint64_t *pre = pre_all + (size_t)t * m;
    uint32_t *lab = lab_all + (size_t)t * n;
    for (uint32_t v = threadIdx.x; v < n; v += NT) par[v] = v;
    if (threadIdx.x == 0) s_count = n;
    __syncthreads();
    const uint64_t seg = (m + NT - 1) / NT;
    const uint64_t lo = min(m, (uint64_t)threadIdx.x * seg), hi = min(m, lo + seg);
    for (uint64_t rnd = 0; s_count > target; rnd++) {
        // weights of the edges that are not loops, and their inclusive prefix in edge order
        uint64_t local = 0;
        for (uint64_t e = lo; e < hi; e++)
            if (par[U[e]] != par[V[e]]) local += Wt[e];
        uint64_t W;
        uint64_t acc = block_excl_scan_u64<NT>(local, W);
        for (uint64_t e = lo; e < hi; e++) {
            if (par[U[e]] != par[V[e]]) acc += Wt[e];
            pre[e] = acc;
        }
        __syncthreads();
        if (W == 0) break;  // the remaining graph has no edges between its vertices
        const uint32_t c_start = s_count;
        for (uint32_t base = 0; base < c_start; base += kBatch) {
            const uint32_t nb = min((uint32_t)kBatch, c_start - base);
            for (uint32_t j = threadIdx.x; j < nb; j += NT) {
                const uint64_t y = mulhi64(draw64(key.k0, key.idx, 1, 0, rnd, base + j), W);
                const uint64_t e = upper_bound_u64(pre, m, y);
                sb[j] = make_uint2(U[e], V[e]);
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                uint32_t c = s_count;
                for (uint32_t j = 0; j < nb && c > target; j++) {
                    const uint32_t a = sfind(par, sb[j].x), b = sfind(par, sb[j].y);
                    if (a != b) {
                        if (a < b) par[b] = a; else par[a] = b;
                        c--;
                    }
                }
                s_count = c;
            }
            __syncthreads();
            if (s_count <= target) break;
        }
        for (uint32_t v = threadIdx.x; v < n; v += NT) par[v] = sfind_ro(par, v);
        __syncthreads();
    }
    rank_labels<NT>(par, n, lab);
    if (threadIdx.x == 0) k_out[t] = s_count;
}

// ---------------------------------------------------------------- stage 2

__global__ void dense_build_kernel(uint64_t m, const uint32_t *__restrict__ U, const uint32_t *__restrict__ V,
                                   const uint32_t *__restrict__ Wt, const uint32_t *__restrict__ lab_all, uint32_t n,
                                   const uint32_t *__restrict__ kdim, const uint64_t *__restrict__ mat_off,
                                   uint64_t *mats) {
    const uint32_t t = blockIdx.y;
    const uint64_t k = kdim[t];
    uint64_t *M = mats + mat_off[t];
    const uint32_t *lab = lab_all ? lab_all + (size_t)t * n : nullptr;
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t a = U[e], b = V[e];
        if (lab) {
            a = lab[a];
            b = lab[b];
        }
        if (a == b) continue;
        const unsigned long long w = Wt[e];
        atomicAdd((unsigned long long *)&M[(uint64_t)a * k + b], w);
        atomicAdd((unsigned long long *)&M[(uint64_t)b * k + a], w);
    }
}

// ---------------------------------------------------------------- stage 3: Karger-Stein

// One warp per matrix row: 32-column block prefixes and the row sum.
__global__ void prep_rows_kernel(const SrcDesc *__restrict__ srcs, const uint64_t *__restrict__ row_off,
                                 uint32_t nsrc, uint64_t total_rows, uint64_t *cuts) {
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
    const uint64_t *row = S.mat + i * S.N;
    uint64_t run = 0;
    for (uint32_t b = 0; b < S.nb; b++) {
        const uint32_t j = b * 32 + lane;
        uint64_t x = j < S.N ? row[j] : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        run += x;
        if (lane == 0) S.blk[i * S.nb + b] = run;
    }
    if (lane == 0) {
        S.rowpre[i] = run;
        if (S.is_root) atomicMin((unsigned long long *)&cuts[S.trial], (unsigned long long)run);
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

template <int NT>
__global__ void __launch_bounds__(NT) contract_kernel(const TaskDesc *__restrict__ tasks,
                                                      const SrcDesc *__restrict__ srcs, uint32_t *__restrict__ k_out,
                                                      uint64_t *cuts, uint32_t *err) {
    extern __shared__ __align__(16) unsigned char dsm[];
    uint2 *sb = reinterpret_cast<uint2 *>(dsm);
    __shared__ uint32_t s_count;
    const TaskDesc T = tasks[blockIdx.x];
    const SrcDesc S = srcs[T.src];
    const uint32_t N = S.N;
    uint32_t *par = reinterpret_cast<uint32_t *>(dsm + kBatch * sizeof(uint2));
    uint32_t *cnt = par + N;  // counting-sort counters, N entries
    const uint64_t W = S.rowpre[N - 1];
    if (W == 0) {  // no edges between the vertices: the cut is 0, nothing to contract
        if (threadIdx.x == 0) {
            k_out[blockIdx.x] = kDropped;
            atomicMin((unsigned long long *)&cuts[T.trial], 0ull);
        }
        return;
    }
    for (uint32_t v = threadIdx.x; v < N; v += NT) par[v] = v;
    if (threadIdx.x == 0) s_count = N;
    __syncthreads();
    for (uint32_t base = 0; base < N; base += kBatch) {
        const uint32_t nb = min((uint32_t)kBatch, N - base);
        for (uint32_t j = threadIdx.x; j < nb; j += NT) {
            const uint64_t y = mulhi64(draw64(T.k0, T.idx, T.tag, 0, T.round, base + j), W);
            const uint32_t a = (uint32_t)upper_bound_u64(S.rowpre, N, y);
            const uint64_t rem = y - (a ? S.rowpre[a - 1] : 0);
            const uint64_t *B = S.blk + (uint64_t)a * S.nb;
            const uint32_t b = (uint32_t)upper_bound_u64(B, S.nb, rem);
            const uint64_t rem2 = rem - (b ? B[b - 1] : 0);
            const uint64_t *row = S.mat + (uint64_t)a * N + (uint64_t)b * 32;
            const uint32_t lim = min(32u, N - b * 32);
            uint64_t acc = 0;
            uint32_t c = 0;
            for (; c < lim; c++) {
                acc += row[c];
                if (acc > rem2) break;
            }
            if (c >= lim) {  // cannot happen with consistent prefixes; record and clamp
                atomicOr(err, 1u);
                c = lim - 1;
            }
            sb[j] = make_uint2(a, b * 32 + c);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t cc = s_count;
            for (uint32_t j = 0; j < nb && cc > T.target; j++) {
                const uint32_t x = sfind(par, sb[j].x), y = sfind(par, sb[j].y);
                if (x != y) {
                    if (x < y) par[y] = x; else par[x] = y;
                    cc--;
                }
            }
            s_count = cc;
        }
        __syncthreads();
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

// One CTA per group of `rows` consecutive output rows of one child. For each row a: the sum of the
// member rows of group a, accumulated column by column in shared memory (each thread owns its
// columns, one pass per member row, coalesced reads); then every output column b gathers its
// members' entries of that sum through the member lists (no atomics). The diagonal (b == a) is 0.
template <int NT>
__global__ void __launch_bounds__(NT) quotient_kernel(const TaskDesc *__restrict__ tasks,
                                                      const SrcDesc *__restrict__ srcs,
                                                      const uint32_t *__restrict__ kdim,
                                                      const uint64_t *__restrict__ group_task_off, uint32_t ntasks,
                                                      uint32_t rows, const uint64_t *__restrict__ out_off,
                                                      uint64_t *out_base) {
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
    const uint32_t N = S.N;
    const uint32_t a0 = (uint32_t)(gg - group_task_off[lo]) * rows, a1 = min(k, a0 + rows);
    uint64_t *rowsum = reinterpret_cast<uint64_t *>(dsm);  // N entries
    uint64_t *Qt = out_base + out_off[lo];
    for (uint32_t a = a0; a < a1; a++) {
        const uint32_t p0 = T.memb_off[a], p1 = T.memb_off[a + 1];
        for (uint32_t p = p0; p < p1; p++) {
            const uint64_t *row = S.mat + (uint64_t)T.members[p] * N;
            if (p == p0) {
                for (uint32_t j = threadIdx.x; j < N; j += NT) rowsum[j] = row[j];
            } else {
                for (uint32_t j = threadIdx.x; j < N; j += NT) rowsum[j] += row[j];
            }
        }
        __syncthreads();
        uint64_t *Q = Qt + (uint64_t)a * k;
        for (uint32_t b = threadIdx.x; b < k; b += NT) {
            uint64_t acc = 0;
            if (b != a) {
                const uint32_t q1 = T.memb_off[b + 1];
                for (uint32_t q = T.memb_off[b]; q < q1; q++) acc += rowsum[T.members[q]];
            }
            Q[b] = acc;
        }
        __syncthreads();
    }
}

// Exact minimum cut of one leaf (n <= 128) by one warp: maximum-adjacency orderings as in the
// reference's Stoer-Wagner base case (co_mincut_base_case.hpp:52-144), with the Nagamochi-Ono-
// Ibaraki contraction rule (Nagamochi & Ibaraki 1992; Nagamochi, Ono & Ibaraki 1994): when vertex
// w's key reaches q >= lambda while vertex v is scanned, then lambda(v, w) >= q, so the edge (v, w)
// can be contracted without losing any cut below lambda, the best cut value found so far (initially
// the leaf's minimum weighted degree). Every ordering contracts all such certified edges plus the
// last two vertices (the cut of the phase updates lambda), so far fewer orderings are needed than
// the n - 1 of plain Stoer-Wagner; the returned value is the exact minimum cut of the leaf.
//   lane l owns vertices l, l+32, l+64, l+96; argmax by warp reduction of (key << 8 | 255 - v),
//   ties to the smallest vertex; keys stay below 2^56 (total graph weight checked on the host).
//   The full matrix sits in shared memory so that a row read is conflict-free; contractions use a
//   small union-find over vertex slots in shared memory.
__device__ __forceinline__ uint64_t warp_min_u64(uint64_t x) {
    const uint32_t hi = (uint32_t)(x >> 32);
    const uint32_t top = __reduce_min_sync(0xffffffffu, hi);
    const uint32_t lo = __reduce_min_sync(0xffffffffu, hi == top ? (uint32_t)x : 0xFFFFFFFFu);
    return ((uint64_t)top << 32) | lo;
}

template <typename Tm>
__global__ void __launch_bounds__(32) sw_leaf_kernel(const LeafDesc *__restrict__ leaves, uint64_t *cuts) {
    extern __shared__ __align__(16) unsigned char dsm[];
    Tm *M = reinterpret_cast<Tm *>(dsm);
    __shared__ uint8_t uf[128];
    __shared__ uint32_t pairs[128];
    __shared__ uint32_t npairs;
    const LeafDesc L = leaves[blockIdx.x];
    const uint32_t N = L.N;
    const int lane = threadIdx.x;
    for (uint32_t x = lane; x < N * N; x += 32) M[x] = (Tm)L.mat[x];
    for (uint32_t x = lane; x < 128; x += 32) uf[x] = (uint8_t)x;
    __syncwarp();
    uint32_t active = 0;
#pragma unroll
    for (int s = 0; s < 4; s++)
        if ((uint32_t)(lane + 32 * s) < N) active |= 1u << s;
    // lambda starts at the minimum weighted degree (a cut of the leaf)
    uint64_t deg_min = kU64Max;
#pragma unroll
    for (int s = 0; s < 4; s++) {
        if ((active >> s) & 1u) {
            const Tm *row = M + (size_t)(lane + 32 * s) * N;
            uint64_t d = 0;
            for (uint32_t x = 0; x < N; x++) d += (uint64_t)row[x];
            deg_min = d < deg_min ? d : deg_min;
        }
    }
    uint64_t lambda = warp_min_u64(deg_min);
    uint32_t cnt = N;
    while (cnt > 1) {
        uint64_t key[4] = {0, 0, 0, 0};
        uint32_t in_a = 0;
        uint32_t mark[4] = {0xFFu, 0xFFu, 0xFFu, 0xFFu};  // vertex to contract into, 0xFF: none
        uint32_t prev = 0, last = 0;
        uint64_t cut_phase = 0;
        for (uint32_t step = 0; step < cnt; step++) {
            uint64_t local = 0;
#pragma unroll
            for (int s = 0; s < 4; s++) {
                if (((active & ~in_a) >> s) & 1u) {
                    const uint64_t cand = (key[s] << 8) | (uint64_t)(255 - (lane + 32 * s));
                    local = cand > local ? cand : local;
                }
            }
            const uint32_t hi = (uint32_t)(local >> 32);
            const uint32_t top = __reduce_max_sync(0xffffffffu, hi);
            const uint32_t lo = __reduce_max_sync(0xffffffffu, hi == top ? (uint32_t)local : 0u);
            local = ((uint64_t)top << 32) | lo;
            const uint32_t sv = 255u - (uint32_t)(local & 255u);
            if (step + 1 == cnt) {
                last = sv;
                cut_phase = local >> 8;
                break;
            }
            if ((uint32_t)lane == (sv & 31u)) in_a |= 1u << (sv >> 5);
            prev = sv;
            const Tm *row = M + (size_t)sv * N;
#pragma unroll
            for (int s = 0; s < 4; s++) {
                if (((active & ~in_a) >> s) & 1u) {
                    const uint64_t c = (uint64_t)row[lane + 32 * s];
                    if (c) {
                        key[s] += c;
                        if (key[s] >= lambda) mark[s] = sv;  // lambda(sv, v) >= key: contractible
                    }
                }
            }
        }
        lambda = cut_phase < lambda ? cut_phase : lambda;
        // contraction list: (prev, last), then every certified edge (v, mark[v])
        if (lane == 0) {
            pairs[0] = (prev << 8) | last;
            npairs = 1;
        }
        __syncwarp();
#pragma unroll
        for (int s = 0; s < 4; s++) {
            const bool has = ((active >> s) & 1u) && mark[s] != 0xFFu;
            const uint32_t bal = __ballot_sync(0xffffffffu, has);
            const uint32_t base = npairs;
            if (has) pairs[base + __popc(bal & ((1u << lane) - 1u))] = (mark[s] << 8) | (uint32_t)(lane + 32 * s);
            __syncwarp();
            if (lane == 0) npairs = base + __popc(bal);
            __syncwarp();
        }
        const uint32_t np = npairs;
        for (uint32_t q = 0; q < np && cnt > 1; q++) {
            uint32_t x = pairs[q] >> 8, y = pairs[q] & 255u;
            while (uf[x] != x) x = uf[x];
            while (uf[y] != y) y = uf[y];
            if (x == y) continue;  // already merged (warp-uniform)
            // merge y into x: entry (x, v) += entry (y, v) for every other active v, both halves
            Tm *rx = M + (size_t)x * N;
            const Tm *ry = M + (size_t)y * N;
#pragma unroll
            for (int s = 0; s < 4; s++) {
                const uint32_t v = lane + 32 * s;
                if (((active >> s) & 1u) && v != x && v != y) {
                    const Tm val = rx[v] + ry[v];
                    rx[v] = val;
                    M[(size_t)v * N + x] = val;
                }
            }
            if ((uint32_t)lane == (y & 31u)) active &= ~(1u << (y >> 5));
            __syncwarp();
            if (lane == 0) uf[y] = (uint8_t)x;
            __syncwarp();
            cnt--;
        }
    }
    if (lane == 0) atomicMin((unsigned long long *)&cuts[L.trial], (unsigned long long)lambda);
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

template <typename T>
int upload(cac_ctx *ctx, DevBuf &buf, const std::vector<T> &v) {
    CAC_TRY(buf.ensure(sizeof(T) * std::max<size_t>(v.size(), 1)));
    if (!v.empty())
        CAC_CUDA_TRY(cudaMemcpyAsync(buf.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, ctx->stream));
    return CAC_OK;
}

struct Node {
    uint32_t trial;  // slot in this wave
    uint64_t h;      // heap index
    uint32_t N;
    uint64_t off;    // element offset of the matrix in the level buffer it lives in
    uint32_t is_root;
};

struct PendingTask {
    uint32_t trial;
    uint64_t h;       // heap index of the child being built
    uint32_t round;
    uint32_t target;
    uint32_t src;     // index into this iteration's source list
};


size_t contract_smem(uint32_t N) { return kBatch * sizeof(uint2) + (size_t)2 * N * 4; }
size_t quotient_smem(uint32_t k, uint32_t N) { return (size_t)N * 8; }

// Runs Stage 3 for the root matrices of one wave; cuts[] (wave slots) must hold the Stage-1/2
// bounds (UINT64_MAX before the root nodes' minimum-degree bound is applied).
int ks_levels(cac_ctx *ctx, std::vector<Node> nodes, DevBuf *cur, DevBuf *next, const std::vector<TrialKey> &keys,
              uint64_t *d_cuts, bool small_entries, uint32_t *d_err) {
    cudaStream_t s = ctx->stream;
    DevBuf d_src(ctx), d_task(ctx), d_leaf(ctx), d_rowoff(ctx), d_kout(ctx), d_prep(ctx), d_tscratch(ctx),
        d_qoff(ctx), d_rto(ctx);
    std::vector<PendingTask> carried;      // tasks continuing with another round (sources in `cur`)
    std::vector<Node> carried_src;         // their source matrices
    while (!nodes.empty() || !carried.empty()) {
        // leaves -> Stoer-Wagner
        std::vector<LeafDesc> leaves;
        std::vector<Node> inner;
        for (const Node &nd : nodes) {
            if (nd.N <= 128) {
                if (nd.N >= 2) leaves.push_back(LeafDesc{cur->as<uint64_t>() + nd.off, nd.N, nd.trial});
            } else {
                inner.push_back(nd);
            }
        }
        if (!leaves.empty()) {
            // group by size so that each launch uses one dynamic shared-memory size
            std::sort(leaves.begin(), leaves.end(), [](const LeafDesc &a, const LeafDesc &b) { return a.N > b.N; });
            CAC_TRY(upload(ctx, d_leaf, leaves));
            size_t first = 0;
            while (first < leaves.size()) {
                size_t last = first;
                while (last < leaves.size() && leaves[last].N == leaves[first].N) last++;
                const uint32_t N = leaves[first].N;
                const LeafDesc *dl = d_leaf.as<LeafDesc>() + first;
                if (small_entries) {
                    const size_t sm = (size_t)N * N * 4;
                    CAC_CUDA_TRY(cudaFuncSetAttribute(sw_leaf_kernel<uint32_t>,
                                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
                    sw_leaf_kernel<uint32_t><<<(unsigned)(last - first), 32, sm, s>>>(dl, d_cuts);
                } else {
                    const size_t sm = (size_t)N * N * 8;
                    CAC_CUDA_TRY(cudaFuncSetAttribute(sw_leaf_kernel<uint64_t>,
                                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
                    sw_leaf_kernel<uint64_t><<<(unsigned)(last - first), 32, sm, s>>>(dl, d_cuts);
                }
                first = last;
            }
            CAC_CUDA_TRY(cudaGetLastError());
        }
        // sources of this iteration: inner nodes (children 0 and 1) + matrices of carried tasks
        std::vector<SrcDesc> srcs;
        std::vector<PendingTask> tasks;
        std::vector<uint64_t> row_off;
        uint64_t rows = 0, prep_elems = 0;
        std::vector<const Node *> src_nodes;
        for (const Node &nd : inner) src_nodes.push_back(&nd);
        for (const Node &nd : carried_src) src_nodes.push_back(&nd);
        for (size_t i = 0; i < src_nodes.size(); i++) {
            const Node &nd = *src_nodes[i];
            const uint32_t nb = (nd.N + 31) / 32;
            prep_elems += nd.N + (uint64_t)nd.N * nb;
        }
        if (src_nodes.empty()) break;
        CAC_TRY(d_prep.ensure(prep_elems * 8));
        uint64_t pe = 0, tscratch = 0;
        for (size_t i = 0; i < src_nodes.size(); i++) {
            const Node &nd = *src_nodes[i];
            SrcDesc S;
            S.mat = cur->as<uint64_t>() + nd.off;
            S.N = nd.N;
            S.nb = (nd.N + 31) / 32;
            S.rowpre = d_prep.as<uint64_t>() + pe;
            S.blk = S.rowpre + nd.N;
            pe += nd.N + (uint64_t)nd.N * S.nb;
            S.trial = nd.trial;
            S.is_root = nd.is_root;
            srcs.push_back(S);
            row_off.push_back(rows);
            rows += nd.N;
        }
        for (size_t i = 0; i < inner.size(); i++) {
            const uint32_t target = (uint32_t)ks_target((int)inner[i].N);
            for (uint64_t c = 0; c < 2; c++)
                tasks.push_back(PendingTask{inner[i].trial, 2 * inner[i].h + c, 0, target, (uint32_t)i});
        }
        for (size_t i = 0; i < carried.size(); i++) {
            PendingTask t = carried[i];
            t.src = (uint32_t)(inner.size() + i);
            tasks.push_back(t);
        }
        for (const PendingTask &t : tasks) tscratch += 2 * (uint64_t)srcs[t.src].N + srcs[t.src].N + 1;
        CAC_TRY(upload(ctx, d_src, srcs));
        CAC_TRY(upload(ctx, d_rowoff, row_off));
        {
            const uint64_t threads = rows * 32;
            const unsigned grid = (unsigned)((threads + 255) / 256);
            prep_rows_kernel<<<grid, 256, 0, s>>>(d_src.as<SrcDesc>(), d_rowoff.as<uint64_t>(),
                                                  (uint32_t)srcs.size(), rows, d_cuts);
            prefix_rows_kernel<kNT><<<(unsigned)srcs.size(), kNT, 0, s>>>(d_src.as<SrcDesc>());
        }
        // contraction tasks
        CAC_TRY(d_tscratch.ensure(tscratch * 4));
        std::vector<TaskDesc> td(tasks.size());
        uint64_t ts = 0;
        uint32_t maxN = 0;
        for (size_t i = 0; i < tasks.size(); i++) {
            const PendingTask &t = tasks[i];
            const uint32_t N = srcs[t.src].N;
            maxN = std::max(maxN, N);
            TaskDesc &d = td[i];
            d.tag = 1 + t.h;
            d.src = t.src;
            d.target = t.target;
            d.round = t.round;
            d.trial = t.trial;
            d.k0 = keys[t.trial].k0;
            d.idx = keys[t.trial].idx;
            d.lab = d_tscratch.as<uint32_t>() + ts;
            d.members = d.lab + N;
            d.memb_off = d.members + N;
            ts += 2 * (uint64_t)N + N + 1;
        }
        CAC_TRY(upload(ctx, d_task, td));
        CAC_TRY(d_kout.ensure(tasks.size() * 4));
        {
            const size_t sm = contract_smem(maxN);
            CAC_CUDA_TRY(cudaFuncSetAttribute(contract_kernel<kNT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)sm));
            contract_kernel<kNT><<<(unsigned)tasks.size(), kNT, sm, s>>>(d_task.as<TaskDesc>(), d_src.as<SrcDesc>(),
                                                                         d_kout.as<uint32_t>(), d_cuts, d_err);
            CAC_CUDA_TRY(cudaGetLastError());
        }
        std::vector<uint32_t> kk(tasks.size());
        CAC_CUDA_TRY(cudaMemcpyAsync(kk.data(), d_kout.p, tasks.size() * 4, cudaMemcpyDeviceToHost, s));
        CAC_CUDA_TRY(cudaStreamSynchronize(s));
        // output matrices of this iteration
        std::vector<uint64_t> out_off(tasks.size(), 0), group_task_off(tasks.size(), 0);
        std::vector<uint32_t> kq(tasks.size(), 0);
        uint64_t out_elems = 0, groups = 0;
        size_t qsm = 0;
        // rows per quotient CTA: one for wide matrices, up to 16 as rows get short
        const uint32_t qrows = std::max<uint32_t>(1, std::min<uint32_t>(16, 4096 / std::max<uint32_t>(maxN, 1)));
        for (size_t i = 0; i < tasks.size(); i++) {
            const uint32_t k = kk[i] == kDropped ? 0 : kk[i];
            kq[i] = k;
            out_off[i] = out_elems;
            group_task_off[i] = groups;
            out_elems += (uint64_t)k * k;
            groups += (k + qrows - 1) / qrows;
            if (k) qsm = std::max(qsm, quotient_smem(k, srcs[tasks[i].src].N));
        }
        CAC_TRY(next->ensure(std::max<uint64_t>(out_elems, 1) * 8));
        if (groups) {
            CAC_TRY(upload(ctx, d_qoff, out_off));
            CAC_TRY(upload(ctx, d_rto, group_task_off));
            CAC_TRY(d_kout.ensure(tasks.size() * 4));
            CAC_CUDA_TRY(cudaMemcpyAsync(d_kout.p, kq.data(), tasks.size() * 4, cudaMemcpyHostToDevice, s));
            CAC_CUDA_TRY(cudaFuncSetAttribute(quotient_kernel<kQT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)qsm));
            quotient_kernel<kQT><<<(unsigned)groups, kQT, qsm, s>>>(
                d_task.as<TaskDesc>(), d_src.as<SrcDesc>(), d_kout.as<uint32_t>(), d_rto.as<uint64_t>(),
                (uint32_t)tasks.size(), qrows, d_qoff.as<uint64_t>(), next->as<uint64_t>());
            CAC_CUDA_TRY(cudaGetLastError());
        }
        CAC_CUDA_TRY(cudaStreamSynchronize(s));
        // next iteration
        std::vector<Node> next_nodes;
        std::vector<PendingTask> next_carried;
        std::vector<Node> next_carried_src;
        for (size_t i = 0; i < tasks.size(); i++) {
            const uint32_t k = kq[i];
            if (k == 0) continue;  // dropped: the source had no edges, its cut 0 is recorded
            Node nd{tasks[i].trial, tasks[i].h, k, out_off[i], 0};
            if (k <= tasks[i].target) {
                next_nodes.push_back(nd);
            } else {
                PendingTask t = tasks[i];
                t.round += 1;
                next_carried.push_back(t);
                next_carried_src.push_back(nd);
            }
        }
        std::swap(cur, next);
        nodes.swap(next_nodes);
        carried.swap(next_carried);
        carried_src.swap(next_carried_src);
    }
    CAC_CUDA_TRY(cudaStreamSynchronize(s));
    return CAC_OK;
}

}  // namespace

int mincut_trials(cac_ctx *ctx, const cac_graph *g, uint32_t seed, uint32_t ranks, uint32_t per_rank,
                  uint64_t *d_cuts, float *device_ms) {
    cudaStream_t s = ctx->stream;
    const uint32_t n = g->n;
    const uint64_t m = g->m;
    const uint64_t R = (uint64_t)ranks * per_rank;
    if (g->total_weight >= (1ull << 55)) {
        set_error("total edge weight >= 2^55 is not supported by the Stoer-Wagner leaf kernel");
        return CAC_ERR_UNSUPPORTED;
    }
    const uint32_t t = intermediate_size(n, m);
    if (t < n && n > kMaxSmemVertices) {
        set_error("graphs with more than 16384 vertices that need sparse pre-contraction are not supported yet");
        return CAC_ERR_UNSUPPORTED;
    }
    if (t > kMaxSmemVertices) {
        set_error("contracted graphs with more than 16384 vertices are not supported yet");
        return CAC_ERR_UNSUPPORTED;
    }
    const bool small_entries = g->total_weight < (1ull << 32);
    CAC_CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
    fill_u64<<<std::max<unsigned>(1, (unsigned)std::min<uint64_t>((R + 255) / 256, 4096)), 256, 0, s>>>(d_cuts, R,
                                                                                                       kU64Max);
    std::vector<TrialKey> all(R);
    for (uint32_t r = 0; r < ranks; r++)
        for (uint32_t i = 0; i < per_rank; i++) all[(uint64_t)r * per_rank + i] = TrialKey{seed + r, i};

    // wave size: trials whose Stage-1 scratch and three levels of matrices fit the budget
    const uint64_t per_trial = (t < n ? 8 * m + 4 * (uint64_t)n : 0) + 3 * 8 * (uint64_t)t * t + 64;
    const uint64_t budget = ctx->budget ? ctx->budget / 2 : (24ull << 30);
    const uint64_t wave = std::max<uint64_t>(1, std::min<uint64_t>({R, budget / per_trial, (uint64_t)65535}));

    DevBuf d_keys(ctx), d_pre(ctx), d_lab(ctx), d_k(ctx), d_moff(ctx), bufA(ctx), bufB(ctx), d_err(ctx);
    CAC_TRY(d_err.ensure(4));
    CAC_CUDA_TRY(cudaMemsetAsync(d_err.p, 0, 4, s));
    for (uint64_t w0 = 0; w0 < R; w0 += wave) {
        const uint32_t B = (uint32_t)std::min<uint64_t>(wave, R - w0);
        std::vector<TrialKey> keys(all.begin() + w0, all.begin() + w0 + B);
        CAC_TRY(upload(ctx, d_keys, keys));
        std::vector<uint32_t> kdim(B, n);
        CAC_TRY(d_k.ensure((size_t)B * 4));
        const uint32_t *lab_ptr = nullptr;
        if (t < n) {
            CAC_TRY(d_pre.ensure((size_t)B * std::max<uint64_t>(m, 1) * 8));
            CAC_TRY(d_lab.ensure((size_t)B * n * 4));
            const size_t sm = kBatch * sizeof(uint2) + (size_t)n * 4;
            CAC_CUDA_TRY(cudaFuncSetAttribute(iss_shrink_kernel<kNT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)sm));
            iss_shrink_kernel<kNT><<<B, kNT, sm, s>>>(n, m, g->u, g->v, g->w, t, d_keys.as<TrialKey>(),
                                                       d_pre.as<uint64_t>(), d_lab.as<uint32_t>(), d_k.as<uint32_t>());
            CAC_CUDA_TRY(cudaGetLastError());
            CAC_CUDA_TRY(cudaMemcpyAsync(kdim.data(), d_k.p, (size_t)B * 4, cudaMemcpyDeviceToHost, s));
            CAC_CUDA_TRY(cudaStreamSynchronize(s));
            lab_ptr = d_lab.as<uint32_t>();
        } else {
            CAC_CUDA_TRY(cudaMemcpyAsync(d_k.p, kdim.data(), (size_t)B * 4, cudaMemcpyHostToDevice, s));
        }
        std::vector<uint64_t> moff(B);
        uint64_t elems = 0;
        std::vector<Node> roots;
        for (uint32_t b = 0; b < B; b++) {
            moff[b] = elems;
            elems += (uint64_t)kdim[b] * kdim[b];
            if (kdim[b] >= 2) roots.push_back(Node{b, 1, kdim[b], moff[b], 1});
            else fill_u64<<<1, 32, 0, s>>>(d_cuts + w0 + b, 1, 0);  // a single vertex left: no cut edge
        }
        CAC_TRY(upload(ctx, d_moff, moff));
        CAC_TRY(bufA.ensure(std::max<uint64_t>(elems, 1) * 8));
        CAC_CUDA_TRY(cudaMemsetAsync(bufA.p, 0, elems * 8, s));
        if (m) {
            dim3 grid((unsigned)std::min<uint64_t>((m + 255) / 256, std::max(1, 4 * ctx->num_sms / (int)std::min<uint32_t>(B, 64u) + 1)), B);
            dense_build_kernel<<<grid, 256, 0, s>>>(m, g->u, g->v, g->w, lab_ptr, n, d_k.as<uint32_t>(),
                                                    d_moff.as<uint64_t>(), bufA.as<uint64_t>());
            CAC_CUDA_TRY(cudaGetLastError());
        }
        CAC_TRY(ks_levels(ctx, roots, &bufA, &bufB, keys, d_cuts + w0, small_entries, d_err.as<uint32_t>()));
    }
    uint32_t err = 0;
    CAC_CUDA_TRY(cudaMemcpyAsync(&err, d_err.p, 4, cudaMemcpyDeviceToHost, s));
    CAC_CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
    CAC_CUDA_TRY(cudaStreamSynchronize(s));
    if (device_ms) CAC_CUDA_TRY(cudaEventElapsedTime(device_ms, ctx->ev[0], ctx->ev[1]));
    if (err) {
        set_error("inconsistent selection prefix in the contraction kernel");
        return CAC_ERR_CUDA;
    }
    return CAC_OK;
}

int ks_dense_one(cac_ctx *ctx, uint32_t n, const uint64_t *mat_host, uint32_t seed, uint32_t rank, uint32_t trial,
                 uint64_t *cut) {
    if (n > kMaxSmemVertices) {
        set_error("dense Karger-Stein supports at most 16384 vertices");
        return CAC_ERR_UNSUPPORTED;
    }
    uint64_t total = 0;
    for (uint64_t i = 0; i < (uint64_t)n * n; i++) total += mat_host[i];
    if (total / 2 >= (1ull << 55)) {
        set_error("total edge weight >= 2^55 is not supported");
        return CAC_ERR_UNSUPPORTED;
    }
    cudaStream_t s = ctx->stream;
    DevBuf bufA(ctx), bufB(ctx), d_cuts(ctx), d_err(ctx);
    CAC_TRY(bufA.ensure((size_t)n * n * 8));
    CAC_TRY(d_cuts.ensure(8));
    CAC_TRY(d_err.ensure(4));
    CAC_CUDA_TRY(cudaMemcpyAsync(bufA.p, mat_host, (size_t)n * n * 8, cudaMemcpyHostToDevice, s));
    CAC_CUDA_TRY(cudaMemsetAsync(d_err.p, 0, 4, s));
    fill_u64<<<1, 32, 0, s>>>(d_cuts.as<uint64_t>(), 1, kU64Max);
    std::vector<TrialKey> keys{TrialKey{seed + rank, trial}};
    std::vector<Node> roots{Node{0, 1, n, 0, 1}};
    CAC_TRY(ks_levels(ctx, roots, &bufA, &bufB, keys, d_cuts.as<uint64_t>(), total / 2 < (1ull << 32),
                      d_err.as<uint32_t>()));
    uint32_t err = 0;
    CAC_CUDA_TRY(cudaMemcpyAsync(cut, d_cuts.p, 8, cudaMemcpyDeviceToHost, s));
    CAC_CUDA_TRY(cudaMemcpyAsync(&err, d_err.p, 4, cudaMemcpyDeviceToHost, s));
    CAC_CUDA_TRY(cudaStreamSynchronize(s));
    if (err) {
        set_error("inconsistent selection prefix in the contraction kernel");
        return CAC_ERR_CUDA;
    }
    return CAC_OK;
}

int exact_small(cac_ctx *ctx, uint32_t n, const uint64_t *mat_host, uint64_t *cut) {
    uint64_t total = 0;
    for (uint64_t i = 0; i < (uint64_t)n * n; i++) total += mat_host[i];
    if (total / 2 >= (1ull << 55)) {
        set_error("total edge weight >= 2^55 is not supported");
        return CAC_ERR_UNSUPPORTED;
    }
    cudaStream_t s = ctx->stream;
    DevBuf buf(ctx), d_cuts(ctx), d_leaf(ctx);
    CAC_TRY(buf.ensure((size_t)n * n * 8));
    CAC_TRY(d_cuts.ensure(8));
    CAC_CUDA_TRY(cudaMemcpyAsync(buf.p, mat_host, (size_t)n * n * 8, cudaMemcpyHostToDevice, s));
    fill_u64<<<1, 32, 0, s>>>(d_cuts.as<uint64_t>(), 1, kU64Max);
    std::vector<LeafDesc> leaves{LeafDesc{buf.as<uint64_t>(), n, 0}};
    CAC_TRY(upload(ctx, d_leaf, leaves));
    if (total / 2 < (1ull << 32)) {
        const size_t sm = (size_t)n * n * 4;
        CAC_CUDA_TRY(cudaFuncSetAttribute(sw_leaf_kernel<uint32_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)sm));
        sw_leaf_kernel<uint32_t><<<1, 32, sm, s>>>(d_leaf.as<LeafDesc>(), d_cuts.as<uint64_t>());
    } else {
        const size_t sm = (size_t)n * n * 8;
        CAC_CUDA_TRY(cudaFuncSetAttribute(sw_leaf_kernel<uint64_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)sm));
        sw_leaf_kernel<uint64_t><<<1, 32, sm, s>>>(d_leaf.as<LeafDesc>(), d_cuts.as<uint64_t>());
    }
    CAC_CUDA_TRY(cudaGetLastError());
    CAC_CUDA_TRY(cudaMemcpyAsync(cut, d_cuts.p, 8, cudaMemcpyDeviceToHost, s));
    CAC_CUDA_TRY(cudaStreamSynchronize(s));
    return CAC_OK;
}

}  // namespace cac
