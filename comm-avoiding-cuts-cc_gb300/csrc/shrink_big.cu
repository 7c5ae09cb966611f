// Stage 1 of square_root trials on graphs with more than 16384 vertices (the union-find no longer
// fits one SM's shared memory). Same trial rule as iss_shrink_kernel in mincut.cu and as the
// reference's SequentialSquareRootCut::iteratedSampling (src/SequentialSquareRootCut.cpp:21-67):
// rounds of (vertex count) weighted draws over the edges that are not loops at the start of the
// round, contracted in draw order until exactly `target` vertices remain, vertices renamed to the
// rank of their smallest member. Here every trial of a chunk runs as grid-wide kernels over
// global memory:
//   big_edge_tiles   per 1024-edge tile: non-loop weights, their inclusive prefix inside the tile
//                    and the tile total (u, v, w read as 16-byte vectors)
//   big_tile_scan    per trial: inclusive prefix of the tile totals -> the round's total weight
//   big_draws        per draw: the selected edge by a binary search over the tile prefix, then
//                    inside the tile
//   big_link         draws [lo, mid) linked concurrently into the union-find (CAS of the larger
//                    root onto the smaller, finds without compression), every link logged; a
//                    successful CAS always joins two components, so the link count is the exact
//                    drop of the vertex count
//   big_decide       per trial: keep the links if the count stays above target, otherwise undo
//                    them; bisection over the draw prefix finds the draw at which the sequential
//                    rule stops (the first attempt is the whole round, which is kept in every
//                    round but the last)
//   big_undo / big_apply_one   undo logged links; apply the single stopping draw
//   big_compress     every vertex points at its root (roots are component minima)
//   big_root_count / big_vscan / big_label_roots / big_label_rest   rank-of-minimum labels
// The host steps rounds until every trial is done (its count reached target, or no edge is left
// between its vertices); a fixed number of bisection iterations per round is enough because each
// one halves the open draw range.
#include "cac_internal.h"
#include "sitmo.cuh"

#include <algorithm>
#include <vector>

namespace cac {
namespace {

constexpr int kBT = 256;         // threads per block
constexpr uint32_t kET = 1024;   // edges per tile (4 per thread)
constexpr uint32_t kVT = 1024;   // vertices per tile (4 per thread)
constexpr uint32_t kPhaseOpen = 0, kPhaseRoundDone = 2;

// One contraction task: its graph (edge arrays, u32 or u64 weights), target, stream key and scratch.
struct BigTrial {
    const uint32_t *U, *V;
    const void *W;    // m weights: u32, or u64 when w64
    uint64_t m;
    uint32_t n, target;
    uint32_t etiles, vtiles;
    uint32_t w64;
    uint32_t *par;    // n
    uint64_t *pre;    // m: inclusive prefix of non-loop weights inside each edge tile
    uint64_t *tsum;   // edge tiles: tile totals, then their inclusive prefix
    uint2 *draws;     // n
    uint32_t *log;    // n
    uint32_t *lab;    // n (output)
    uint32_t *vsum;   // vertex tiles: root counts, then exclusive offsets
    uint32_t *k_out;  // output: vertices left
    uint32_t k0, idx; // stream key words 0, 1
    uint64_t tag;     // stream key word 2
    uint32_t dpr;     // draws per round (0: the round's vertex count)
    uint32_t pad;
};

struct BigState {
    uint64_t W;
    uint32_t count, ndraw, lo, hi, mid, nlog, undo_n, apply_one, round, done, phase, err;
};

template <int NT>
__device__ __forceinline__ uint64_t bscan_u64(uint64_t x, uint64_t &total) {
    __shared__ uint64_t ws[NT / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint64_t inc = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) ws[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        uint64_t s = lane < NT / 32 ? ws[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < NT / 32) ws[lane] = s;
    }
    __syncthreads();
    total = ws[NT / 32 - 1];
    const uint64_t off = wid ? ws[wid - 1] : 0;
    __syncthreads();
    return off + inc - x;
}

__device__ __forceinline__ uint64_t ub_u64(const uint64_t *a, uint64_t len, uint64_t y) {
    uint64_t lo = 0, hi = len - 1;  // first i with a[i] > y; a[len - 1] > y
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (a[mid] > y) hi = mid; else lo = mid + 1;
    }
    return lo;
}

__device__ __forceinline__ uint32_t groot(const uint32_t *par, uint32_t x) {
    const volatile uint32_t *vp = par;
    uint32_t p;
    while ((p = vp[x]) != x) x = p;
    return x;
}

__global__ void big_init(const BigTrial *T, BigState *st) {
    const uint32_t b = blockIdx.y;
    const BigTrial &t = T[b];
    uint32_t *par = t.par;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < t.n; v += gridDim.x * blockDim.x) par[v] = v;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        BigState s{};
        s.count = t.n;
        s.done = t.n <= t.target ? 1u : 0u;
        s.phase = kPhaseRoundDone;
        st[b] = s;
    }
}

// Per 1024-edge tile of one task: the weights of its edges that are not loops under the current
// union-find, their inclusive prefix inside the tile and the tile total. The 16-byte vector path
// needs 16-byte aligned arrays (u32 weights; u64 weights are read as two 16-byte halves).
template <bool kW64>
__global__ void __launch_bounds__(kBT) big_edge_tiles(const BigTrial *T, const BigState *st) {
    const uint32_t b = blockIdx.y;
    const BigTrial &t = T[b];
    if (st[b].done || blockIdx.x >= t.etiles || (t.w64 != 0) != kW64) return;
    const uint32_t *par = t.par;
    const uint64_t e0 = (uint64_t)blockIdx.x * kET + threadIdx.x * 4;
    uint32_t u[4], v[4];
    uint64_t w[4];
    const bool aligned = ((reinterpret_cast<uintptr_t>(t.U) | reinterpret_cast<uintptr_t>(t.V) |
                           reinterpret_cast<uintptr_t>(t.W)) & 15) == 0;
    if (e0 + 3 < t.m && aligned) {
        const uint4 uu = *reinterpret_cast<const uint4 *>(t.U + e0);
        const uint4 vv = *reinterpret_cast<const uint4 *>(t.V + e0);
        u[0] = uu.x; u[1] = uu.y; u[2] = uu.z; u[3] = uu.w;
        v[0] = vv.x; v[1] = vv.y; v[2] = vv.z; v[3] = vv.w;
        if (kW64) {
            const ulonglong2 w01 = *reinterpret_cast<const ulonglong2 *>(static_cast<const uint64_t *>(t.W) + e0);
            const ulonglong2 w23 = *reinterpret_cast<const ulonglong2 *>(static_cast<const uint64_t *>(t.W) + e0 + 2);
            w[0] = w01.x; w[1] = w01.y; w[2] = w23.x; w[3] = w23.y;
        } else {
            const uint4 ww = *reinterpret_cast<const uint4 *>(static_cast<const uint32_t *>(t.W) + e0);
            w[0] = ww.x; w[1] = ww.y; w[2] = ww.z; w[3] = ww.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const bool in = e0 + k < t.m;
            u[k] = in ? t.U[e0 + k] : 0;
            v[k] = in ? t.V[e0 + k] : 0;
            w[k] = !in ? 0 : kW64 ? static_cast<const uint64_t *>(t.W)[e0 + k] : static_cast<const uint32_t *>(t.W)[e0 + k];
        }
    }
    uint64_t x[4], local = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        x[k] = (w[k] && par[u[k]] != par[v[k]]) ? w[k] : 0;
        local += x[k];
    }
    uint64_t tot;
    uint64_t acc = bscan_u64<kBT>(local, tot);
    uint64_t *pre = t.pre;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        acc += x[k];
        if (e0 + k < t.m) pre[e0 + k] = acc;
    }
    if (threadIdx.x == 0) t.tsum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) big_tile_scan(const BigTrial *T, BigState *st) {
    const uint32_t b = blockIdx.x;
    if (st[b].done) return;
    const BigTrial &t = T[b];
    uint64_t *ts = t.tsum;
    uint64_t carry = 0;
    for (uint32_t base = 0; base < t.etiles; base += 1024) {
        const uint32_t i = base + threadIdx.x;
        const uint64_t x = i < t.etiles ? ts[i] : 0;
        uint64_t tot;
        const uint64_t ex = bscan_u64<1024>(x, tot);
        if (i < t.etiles) ts[i] = carry + ex + x;
        carry += tot;
    }
    if (threadIdx.x == 0) {
        BigState &s = st[b];
        s.W = carry;
        if (carry == 0) {  // no edge left between the vertices: the trial keeps its count
            s.done = 1;
            s.phase = kPhaseRoundDone;
        } else {
            s.ndraw = t.dpr ? t.dpr : s.count;
            s.lo = 0;
            s.hi = s.ndraw;
            s.mid = s.ndraw;
            s.nlog = 0;
            s.undo_n = 0;
            s.apply_one = 0;
            s.phase = kPhaseOpen;
        }
    }
}

__global__ void __launch_bounds__(kBT) big_draws(const BigTrial *T, const BigState *st) {
    const uint32_t b = blockIdx.y;
    const BigState s = st[b];
    if (s.done) return;
    const BigTrial &t = T[b];
    for (uint32_t j = blockIdx.x * kBT + threadIdx.x; j < s.ndraw; j += gridDim.x * kBT) {
        const uint64_t y = mulhi64(draw64(t.k0, t.idx, t.tag, 0, s.round, j), s.W);
        const uint32_t tile = (uint32_t)ub_u64(t.tsum, t.etiles, y);
        const uint64_t base = tile ? t.tsum[tile - 1] : 0;
        const uint64_t e0 = (uint64_t)tile * kET;
        const uint64_t len = min((uint64_t)kET, t.m - e0);
        const uint64_t e = e0 + ub_u64(t.pre + e0, len, y - base);
        t.draws[j] = make_uint2(t.U[e], t.V[e]);
    }
}

__global__ void __launch_bounds__(kBT) big_link(const BigTrial *T, BigState *st) {
    const uint32_t b = blockIdx.y;
    const BigState s = st[b];
    if (s.done || s.phase != kPhaseOpen) return;
    const BigTrial t = T[b];
    for (uint32_t j = s.lo + blockIdx.x * kBT + threadIdx.x; j < s.mid; j += gridDim.x * kBT) {
        uint32_t x = t.draws[j].x, y = t.draws[j].y;
        for (;;) {
            x = groot(t.par, x);
            y = groot(t.par, y);
            if (x == y) break;
            const uint32_t hi = max(x, y), lo = min(x, y);
            if (atomicCAS(&t.par[hi], hi, lo) == hi) {
                t.log[atomicAdd(&st[b].nlog, 1u)] = hi;
                break;
            }
            x = hi;  // hi was linked meanwhile: find both roots again
            y = lo;
        }
    }
}

__global__ void big_decide(const BigTrial *T, BigState *st, uint32_t B) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const uint32_t target = T[b].target;
    BigState &s = st[b];
    if (s.done || s.phase != kPhaseOpen) return;
    const uint32_t links = s.nlog;
    s.nlog = 0;
    if (s.count - links > target) {  // keep: the sequential rule would not stop inside [lo, mid)
        s.count -= links;
        s.lo = s.mid;
        s.undo_n = 0;
        if (s.lo == s.hi) {
            if (s.hi == s.ndraw) s.phase = kPhaseRoundDone;  // the whole round was applied
            else s.err = 1;  // cannot happen: [lo, hi) is known to reach target
        } else {
            s.mid = s.lo + max(1u, (s.hi - s.lo) / 2);
        }
    } else {  // the stop lies inside [lo, mid): undo, then search the lower half
        s.undo_n = links;
        s.hi = s.mid;
        if (s.hi - s.lo == 1) s.apply_one = 1;  // draw lo alone reaches target
        else s.mid = s.lo + (s.hi - s.lo) / 2;
    }
}

__global__ void __launch_bounds__(kBT) big_undo(const BigTrial *T, const BigState *st) {
    const uint32_t b = blockIdx.y;
    const uint32_t n = st[b].undo_n;
    if (!n) return;
    const BigTrial t = T[b];
    for (uint32_t i = blockIdx.x * kBT + threadIdx.x; i < n; i += gridDim.x * kBT) t.par[t.log[i]] = t.log[i];
}

__global__ void big_apply_one(const BigTrial *T, BigState *st, uint32_t B) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const uint32_t target = T[b].target;
    BigState &s = st[b];
    s.undo_n = 0;
    if (!s.apply_one) return;
    s.apply_one = 0;
    const BigTrial t = T[b];
    const uint32_t x = groot(t.par, t.draws[s.lo].x), y = groot(t.par, t.draws[s.lo].y);
    if (x != y) {
        t.par[max(x, y)] = min(x, y);
        s.count -= 1;
    }
    if (s.count != target) s.err = 1;  // cannot happen: this draw was shown to reach target
    s.done = 1;
    s.phase = kPhaseRoundDone;
}

__global__ void big_compress(const BigTrial *T) {
    const uint32_t b = blockIdx.y;
    uint32_t *par = T[b].par;
    const uint32_t n = T[b].n;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        par[v] = groot(par, v);
}

__global__ void big_round_end(const BigTrial *T, BigState *st, uint32_t B, uint32_t *active) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const uint32_t target = T[b].target;
    BigState &s = st[b];
    if (!s.done && s.phase != kPhaseRoundDone) s.err = 1;  // bisection did not close
    s.round += 1;
    if (s.count <= target) s.done = 1;
    if (!s.done) atomicAdd(active, 1u);
}

__global__ void __launch_bounds__(kBT) big_root_count(const BigTrial *T) {
    const uint32_t b = blockIdx.y;
    if (blockIdx.x >= T[b].vtiles) return;
    const uint32_t *par = T[b].par;
    const uint32_t n = T[b].n;
    const uint32_t v0 = blockIdx.x * kVT + threadIdx.x * 4;
    uint32_t c = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) c += (v0 + k < n && par[v0 + k] == v0 + k) ? 1u : 0u;
    c = __reduce_add_sync(0xffffffffu, c);
    __shared__ uint32_t ws[kBT / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t s = 0;
        for (int i = 0; i < kBT / 32; i++) s += ws[i];
        T[b].vsum[blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(1024) big_vscan(const BigTrial *T) {
    const uint32_t b = blockIdx.x;
    uint32_t *vs = T[b].vsum;
    const uint32_t vtiles = T[b].vtiles;
    uint64_t carry = 0;
    for (uint32_t base = 0; base < vtiles; base += 1024) {
        const uint32_t i = base + threadIdx.x;
        const uint64_t x = i < vtiles ? vs[i] : 0;
        uint64_t tot;
        const uint64_t ex = bscan_u64<1024>(x, tot);
        if (i < vtiles) vs[i] = (uint32_t)(carry + ex);
        carry += tot;
    }
    if (threadIdx.x == 0) *T[b].k_out = (uint32_t)carry;
}

__global__ void __launch_bounds__(kBT) big_label_roots(const BigTrial *T) {
    const uint32_t b = blockIdx.y;
    const BigTrial &t = T[b];
    if (blockIdx.x >= t.vtiles) return;
    const uint32_t v0 = blockIdx.x * kVT + threadIdx.x * 4;
    uint32_t f[4], c = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        f[k] = (v0 + k < t.n && t.par[v0 + k] == v0 + k) ? 1u : 0u;
        c += f[k];
    }
    uint64_t tot;
    uint32_t r = t.vsum[blockIdx.x] + (uint32_t)bscan_u64<kBT>(c, tot);
#pragma unroll
    for (int k = 0; k < 4; k++)
        if (f[k]) t.lab[v0 + k] = r++;
}

__global__ void big_label_rest(const BigTrial *T) {
    const uint32_t b = blockIdx.y;
    const BigTrial &t = T[b];
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < t.n; v += gridDim.x * blockDim.x) {
        const uint32_t r = t.par[v];
        if (r != v) t.lab[v] = t.lab[r];
    }
}

}  // namespace

// Scratch of one contraction task, carved in the order shrink_tasks takes it (dpr: draws per
// round, 0 for the vertex count; the draw list holds a round's draws).
uint64_t shrink_task_scratch(uint32_t n, uint64_t m, uint32_t dpr) {
    const uint64_t etiles = (m + kET - 1) / kET, vtiles = ((uint64_t)n + kVT - 1) / kVT;
    const uint64_t nd = std::max<uint64_t>(n, dpr);
    return align_up(4ull * n) + align_up(8 * std::max<uint64_t>(m, 1)) + align_up(8 * std::max<uint64_t>(etiles, 1)) +
           align_up(8ull * nd) + align_up(4ull * n) + align_up(4 * std::max<uint64_t>(vtiles, 1));
}

uint64_t shrink_tasks_scratch(const std::vector<ShrinkTask> &tasks) {
    uint64_t b = align_up(sizeof(BigTrial) * tasks.size()) + align_up(sizeof(BigState) * tasks.size()) + align_up(16);
    for (const ShrinkTask &t : tasks) b += shrink_task_scratch(t.n, t.m, t.dpr);
    return b;
}

// Stage-1 contraction of every task (rounds of weighted draws over the task's edges that are not
// loops, contracted in draw order until exactly its target is left, or no edge is left), all
// tasks stepped together: labels (rank of the smallest member) to task.lab, vertices left to
// *task.k_out. The tasks may have different graphs, sizes, targets and keys.
int shrink_tasks(cac_ctx *ctx, const std::vector<ShrinkTask> &tasks, void *scratch) {
    cudaStream_t s = ctx->stream;
    const uint32_t B = (uint32_t)tasks.size();
    if (B == 0) return CAC_OK;
    if (B > 65535) {
        set_error("shrink_tasks: more than 65535 tasks in one call");
        return CAC_ERR_INVALID;
    }
    std::vector<BigTrial> T(B);
    char *p = static_cast<char *>(scratch);
    auto take = [&](size_t bytes) {
        char *q = p;
        p += align_up(bytes);
        return q;
    };
    uint32_t nmax = 1, etmax = 1, vtmax = 1, dmax = 1;
    uint64_t mmax = 0;
    bool any32 = false, any64 = false;
    for (uint32_t b = 0; b < B; b++) {
        const ShrinkTask &k = tasks[b];
        BigTrial &t = T[b];
        t.U = k.U;
        t.V = k.V;
        t.W = k.W;
        t.m = k.m;
        t.n = k.n;
        t.target = k.target;
        t.etiles = (uint32_t)((k.m + kET - 1) / kET);
        t.vtiles = (uint32_t)((k.n + kVT - 1) / kVT);
        t.w64 = k.w64 ? 1u : 0u;
        t.par = reinterpret_cast<uint32_t *>(take(4ull * k.n));
        t.pre = reinterpret_cast<uint64_t *>(take(8 * std::max<uint64_t>(k.m, 1)));
        t.tsum = reinterpret_cast<uint64_t *>(take(8ull * std::max<uint32_t>(t.etiles, 1)));
        t.draws = reinterpret_cast<uint2 *>(take(8ull * std::max<uint32_t>(k.n, k.dpr)));
        t.log = reinterpret_cast<uint32_t *>(take(4ull * k.n));
        t.vsum = reinterpret_cast<uint32_t *>(take(4ull * std::max<uint32_t>(t.vtiles, 1)));
        t.lab = k.lab;
        t.k_out = k.k_out;
        t.k0 = k.k0;
        t.idx = k.idx;
        t.tag = k.tag;
        t.dpr = k.dpr;
        t.pad = 0;
        nmax = std::max(nmax, k.n);
        dmax = std::max(dmax, std::max(k.n, k.dpr));
        mmax = std::max(mmax, k.m);
        etmax = std::max(etmax, t.etiles);
        vtmax = std::max(vtmax, t.vtiles);
        (k.w64 ? any64 : any32) = true;
    }
    BigTrial *dT = reinterpret_cast<BigTrial *>(take(sizeof(BigTrial) * B));
    BigState *dS = reinterpret_cast<BigState *>(take(sizeof(BigState) * B));
    uint32_t *d_active = reinterpret_cast<uint32_t *>(take(16));
    CAC_CUDA_TRY(cudaMemcpyAsync(dT, T.data(), sizeof(BigTrial) * B, cudaMemcpyHostToDevice, s));
    const uint32_t vgrid = std::max(1u, std::min<uint32_t>((nmax + kBT - 1) / kBT, 2048u / std::max(1u, B / 8 + 1)));
    big_init<<<dim3(vgrid, B), kBT, 0, s>>>(dT, dS);
    const uint32_t dgrid = std::max(1u, std::min<uint32_t>((dmax + kBT - 1) / kBT, 4096u / B + 1));
    uint32_t iters = 3;
    while ((1ull << (iters - 3)) < dmax) iters++;  // ceil(log2 draws) + 3 bisection steps close every round
    const unsigned tb = (B + 31) / 32;
    for (uint32_t round = 0;; round++) {
        if (round > nmax) {  // every round with edges left links at least its first draw
            set_error("Stage 1: more sampling rounds than vertices");
            return CAC_ERR_CUDA;
        }
        if (mmax) {
            if (any32) big_edge_tiles<false><<<dim3(etmax, B), kBT, 0, s>>>(dT, dS);
            if (any64) big_edge_tiles<true><<<dim3(etmax, B), kBT, 0, s>>>(dT, dS);
            big_tile_scan<<<B, 1024, 0, s>>>(dT, dS);
            big_draws<<<dim3(dgrid, B), kBT, 0, s>>>(dT, dS);
            for (uint32_t it = 0; it < iters; it++) {
                big_link<<<dim3(dgrid, B), kBT, 0, s>>>(dT, dS);
                big_decide<<<tb, 32, 0, s>>>(dT, dS, B);
                big_undo<<<dim3(dgrid, B), kBT, 0, s>>>(dT, dS);
                big_apply_one<<<tb, 32, 0, s>>>(dT, dS, B);
            }
        }
        big_compress<<<dim3(vgrid, B), kBT, 0, s>>>(dT);
        CAC_CUDA_TRY(cudaMemsetAsync(d_active, 0, 4, s));
        big_round_end<<<tb, 32, 0, s>>>(dT, dS, B, d_active);
        CAC_CUDA_TRY(cudaGetLastError());
        uint32_t active = 0;
        CAC_CUDA_TRY(cudaMemcpyAsync(&active, d_active, 4, cudaMemcpyDeviceToHost, s));
        CAC_CUDA_TRY(cudaStreamSynchronize(s));
        if (!active || !mmax) break;
    }
    std::vector<BigState> hs(B);
    CAC_CUDA_TRY(cudaMemcpyAsync(hs.data(), dS, sizeof(BigState) * B, cudaMemcpyDeviceToHost, s));
    CAC_CUDA_TRY(cudaStreamSynchronize(s));
    for (const BigState &x : hs)
        if (x.err) {
            set_error("Stage 1: inconsistent contraction state");
            return CAC_ERR_CUDA;
        }
    big_root_count<<<dim3(vtmax, B), kBT, 0, s>>>(dT);
    big_vscan<<<B, 1024, 0, s>>>(dT);
    big_label_roots<<<dim3(vtmax, B), kBT, 0, s>>>(dT);
    big_label_rest<<<dim3(vgrid, B), kBT, 0, s>>>(dT);
    CAC_CUDA_TRY(cudaGetLastError());
    return CAC_OK;
}

// Scratch of shrink_big for B trials of one graph.
uint64_t shrink_big_scratch(uint32_t n, uint64_t m, uint32_t B) {
    return shrink_task_scratch(n, m, 0) * B + align_up(sizeof(BigTrial) * B) + align_up(sizeof(BigState) * B) +
           align_up(16);
}

int shrink_big(cac_ctx *ctx, const cac_graph *g, uint32_t target, uint32_t B, const uint32_t *k0, const uint32_t *idx,
               uint32_t *d_lab, uint32_t *d_kout, void *scratch) {
    std::vector<ShrinkTask> tasks(B);
    for (uint32_t b = 0; b < B; b++)
        tasks[b] = ShrinkTask{g->u, g->v, g->w, false, g->m, g->n, target, k0[b], idx[b], 1,
                              d_lab + (size_t)b * g->n, d_kout + b, 0};
    return shrink_tasks(ctx, tasks, scratch);
}

}  // namespace cac
