// Device sort and merge of weighted edge lists: the GB300 form of the reference's relabel / sort /
// duplicate-merge step (src/WeightedIteratedSparseSampling.cpp:26-234 with
// src/sorting/SamplingSorter.hpp:44-180, which sample-sort (u, v, w) triples across ranks and then
// sum the weights of equal (u, v); src/karger-stein/sparse_graph.hpp:451-545 relabel + compact).
//
//   edge_keys         relabel: edge (a, b, w) of the parent becomes key lab[a] * k + lab[b] with
//                     the smaller label first, or the loop key k * k when both labels agree
//   radix sort        least-significant-digit, 8-bit digits, stable, (u64 key, u64 weight) pairs:
//                     per pass a per-tile digit histogram, one exclusive scan over (digit, tile),
//                     and a stable scatter that ranks equal digits inside a tile by warp match
//                     voting; only the digits below the key bound are sorted
//   merge             segment heads (key differs from its predecessor), an exclusive scan of the
//                     heads gives each distinct key its slot, and each head sums its segment's
//                     weights in list order into its slot (u64, exact); loop keys are dropped
// The merged list is sorted by (smaller end, larger end) and holds each pair once.
#include "cac_internal.h"

#include <algorithm>

namespace cac {
namespace {

constexpr int kST = 256;                   // threads per sort CTA
constexpr int kSItems = 16;                // keys per thread in a sort tile
constexpr int kSTile = kST * kSItems;      // keys per sort tile
constexpr int kRadix = 256;

// Exclusive scan of n u32 values in place, by tiles of 4096: tile sums, a scan of the sums by one
// CTA (looped), then every tile adds its offset. *total receives the sum.
__global__ void __launch_bounds__(kST) scan_tile_sums(const uint32_t *x, uint64_t n, uint32_t *sums) {
    __shared__ uint32_t ws[kST / 32];
    const uint64_t base = (uint64_t)blockIdx.x * kSTile;
    uint32_t s = 0;
    for (int k = 0; k < kSItems; k++) {
        const uint64_t i = base + (uint64_t)k * kST + threadIdx.x;
        if (i < n) s += x[i];
    }
    s = __reduce_add_sync(0xffffffffu, s);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < kST / 32; w++) t += ws[w];
        sums[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(1024) scan_sums(uint32_t *sums, uint32_t nt, uint32_t *total) {
    __shared__ uint32_t ws[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (uint32_t base = 0; base < nt; base += 1024) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t x = i < nt ? sums[i] : 0;
        uint32_t s = x;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (l >= o) s += y;
        }
        if (l == 31) ws[w] = s;
        __syncthreads();
        if (w == 0) {
            uint32_t t = ws[l];
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
                if (l >= o) t += y;
            }
            ws[l] = t;
        }
        __syncthreads();
        const uint32_t off = carry + (w ? ws[w - 1] : 0);
        if (i < nt) sums[i] = off + s - x;
        __syncthreads();
        if (threadIdx.x == 1023) carry = off + s;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

__global__ void __launch_bounds__(kST) scan_apply(uint32_t *x, uint64_t n, const uint32_t *sums) {
    __shared__ uint32_t ws[kST / 32];
    const uint64_t base = (uint64_t)blockIdx.x * kSTile + (uint64_t)threadIdx.x * kSItems;
    uint32_t v[kSItems], s = 0;
#pragma unroll
    for (int k = 0; k < kSItems; k++) {
        v[k] = base + k < n ? x[base + k] : 0;
        s += v[k];
    }
    const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t inc = s;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (l >= o) inc += y;
    }
    if (l == 31) ws[w] = inc;
    __syncthreads();
    uint32_t before = sums[blockIdx.x];
    for (int i = 0; i < w; i++) before += ws[i];
    uint32_t acc = before + inc - s;
#pragma unroll
    for (int k = 0; k < kSItems; k++) {
        if (base + k < n) x[base + k] = acc;
        acc += v[k];
    }
}

// relabelled keys and weights of a parent's edges (loops get the largest key, k * k)
template <typename WT>
__global__ void edge_keys(const uint32_t *__restrict__ a, const uint32_t *__restrict__ b, const WT *__restrict__ w,
                          uint64_t m, const uint32_t *__restrict__ lab, uint32_t k, uint64_t *keys, uint64_t *vals) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x = a[e], y = b[e];
        if (lab) {
            x = lab[x];
            y = lab[y];
        }
        const uint32_t lo = min(x, y), hi = max(x, y);
        keys[e] = lo == hi ? (uint64_t)k * k : (uint64_t)lo * k + hi;
        vals[e] = (uint64_t)w[e];
    }
}

// per-tile histogram of digit (key >> shift) & 255, stored digit-major: hist[d * tiles + tile]
__global__ void __launch_bounds__(kST) radix_hist(const uint64_t *__restrict__ keys, uint64_t n, int shift,
                                                  uint32_t *hist, uint32_t tiles) {
    __shared__ uint32_t h[kRadix];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * kSTile;
    for (int k = 0; k < kSItems; k++) {
        const uint64_t i = base + (uint64_t)k * kST + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255], 1u);
    }
    __syncthreads();
    hist[(uint64_t)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one tile: rounds of kST keys in order; inside a round, a key's position among
// the equal digits before it = earlier rounds' count + earlier warps' count + its rank in its warp
// (match voting). offs[d * tiles + tile] is where this tile's keys of digit d start.
__global__ void __launch_bounds__(kST) radix_scatter(const uint64_t *__restrict__ keys, const uint64_t *__restrict__ vals,
                                                     uint64_t n, int shift, const uint32_t *__restrict__ offs,
                                                     uint32_t tiles, uint64_t *okeys, uint64_t *ovals) {
    __shared__ uint32_t base[kRadix];
    __shared__ uint32_t wcnt[kST / 32][kRadix];
    const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
    base[threadIdx.x] = offs[(uint64_t)threadIdx.x * tiles + blockIdx.x];
    for (int j = 0; j < kST / 32; j++) wcnt[j][threadIdx.x] = 0;
    __syncthreads();
    const uint64_t t0 = (uint64_t)blockIdx.x * kSTile;
    for (int k = 0; k < kSItems; k++) {
        const uint64_t i = t0 + (uint64_t)k * kST + threadIdx.x;
        const bool in = i < n;
        const uint64_t key = in ? keys[i] : 0;
        const uint64_t val = in ? vals[i] : 0;
        const uint32_t d = in ? (uint32_t)(key >> shift) & 255 : 256u + l;  // off-range lanes match nobody
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t rank = __popc(peers & ((1u << l) - 1));
        if (in && rank == 0) wcnt[w][d] = __popc(peers);
        __syncthreads();
        if (in) {
            uint32_t pos = base[d] + rank;
            for (int j = 0; j < w; j++) pos += wcnt[j][d];
            okeys[pos] = key;
            ovals[pos] = val;
        }
        __syncthreads();
        uint32_t add = 0;
        for (int j = 0; j < kST / 32; j++) {
            add += wcnt[j][threadIdx.x];
            wcnt[j][threadIdx.x] = 0;
        }
        base[threadIdx.x] += add;
        __syncthreads();
    }
}

__global__ void seg_heads(const uint64_t *keys, uint64_t n, uint64_t loop_key, uint32_t *head) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        head[i] = keys[i] != loop_key && (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u;
}

// After the scan, slot[i] is the number of distinct keys before i: the head of every segment of
// equal keys writes its pair and the sum of its segment's weights (read in order from the sorted
// list; no atomics, so heavily merged pairs cost no contention).
__device__ __forceinline__ unsigned long long seg_sum(const uint64_t *keys, const uint64_t *vals, uint64_t n,
                                                      uint64_t i) {
    const uint64_t key = keys[i];
    unsigned long long sum = 0;
    for (uint64_t j = i; j < n && keys[j] == key; j++) sum += vals[j];
    return sum;
}

__global__ void seg_merge(const uint64_t *keys, const uint64_t *vals, uint64_t n, uint64_t loop_key, uint32_t k,
                          const uint32_t *slot, uint32_t *oa, uint32_t *ob, unsigned long long *ow) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t key = keys[i];
        if (key == loop_key || (i > 0 && keys[i - 1] == key)) continue;
        const uint32_t s = slot[i];
        oa[s] = (uint32_t)(key / k);
        ob[s] = (uint32_t)(key % k);
        ow[s] = seg_sum(keys, vals, n, i);
    }
}

// Many children at once: task y writes its edges' keys at in_off, offset by key_off (the sum of the
// earlier tasks' k^2), so one sort orders every task's pairs after the previous task's; loops of
// every task get the one key `loop_key` (= the sum of all k^2), which sorts last.
__global__ void edge_keys_multi(const MergeTask *__restrict__ tasks, uint64_t loop_key, uint64_t *keys,
                                uint64_t *vals) {
    const MergeTask t = tasks[blockIdx.y];
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < t.m; e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x = t.a[e], y = t.b[e];
        if (t.lab) {
            x = t.lab[x];
            y = t.lab[y];
        }
        const uint32_t lo = min(x, y), hi = max(x, y);
        keys[t.in_off + e] = lo == hi ? loop_key : t.key_off + (uint64_t)lo * t.k + hi;
        vals[t.in_off + e] = t.w64 ? static_cast<const uint64_t *>(t.w)[e] : (uint64_t) static_cast<const uint32_t *>(t.w)[e];
    }
}

// The merge of many tasks: as seg_merge, with each head's task found by a binary search over the
// tasks' key ranges.
__global__ void seg_merge_multi(const uint64_t *keys, const uint64_t *vals, uint64_t n, uint64_t loop_key,
                                const MergeTask *__restrict__ tasks, uint32_t ntasks, const uint32_t *slot, uint32_t *oa,
                                uint32_t *ob, unsigned long long *ow) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t key = keys[i];
        if (key == loop_key || (i > 0 && keys[i - 1] == key)) continue;
        const uint32_t s = slot[i];
        uint32_t lo = 0, hi = ntasks - 1;  // last task whose key range starts at or below key
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (tasks[mid].key_off <= key) lo = mid; else hi = mid - 1;
        }
        const uint64_t r = key - tasks[lo].key_off;
        oa[s] = (uint32_t)(r / tasks[lo].k);
        ob[s] = (uint32_t)(r % tasks[lo].k);
        ow[s] = seg_sum(keys, vals, n, i);
    }
}

// first index of the sorted keys[0, n) whose key is >= x
__device__ __forceinline__ uint64_t lower_bound_u64(const uint64_t *keys, uint64_t n, uint64_t x) {
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (keys[mid] < x) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Pairs per task: the keys of task t are the sorted range [key_off[t], key_off[t] + k^2), so its
// pairs are the heads between the two ends of that range: a difference of the heads' exclusive
// scan at two binary-searched positions (no per-head counter, which would make every head of a
// task contend on one word).
__global__ void task_counts(const uint64_t *keys, uint64_t n, const uint32_t *slot, const uint32_t *total,
                            const MergeTask *__restrict__ tasks, uint32_t ntasks, uint32_t *counts) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntasks) return;
    const MergeTask T = tasks[t];
    const uint64_t a = lower_bound_u64(keys, n, T.key_off);
    const uint64_t b = lower_bound_u64(keys, n, T.key_off + (uint64_t)T.k * T.k);
    const uint32_t sa = a < n ? slot[a] : *total, sb = b < n ? slot[b] : *total;
    counts[t] = sb - sa;
}

unsigned grid_of(cac_ctx *ctx, uint64_t work) {
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((work + 255) / 256, (uint64_t)ctx->num_sms * 8));
}

}  // namespace

// Tile sums of scan_u32 over the larger of its two uses here: the digit histogram (256 words per
// tile, 1/16 of a word per key) and the segment heads (one word per key).
uint64_t scan_sum_words(uint64_t m) {
    const uint64_t tiles = (m + kSTile - 1) / kSTile;
    return std::max<uint64_t>(tiles, (kRadix * tiles + kSTile - 1) / kSTile) + 1;
}

uint64_t merge_edges_scratch(uint64_t m) {
    const uint64_t tiles = (m + kSTile - 1) / kSTile;
    return 4 * align_up(8 * std::max<uint64_t>(m, 1)) + align_up(4 * kRadix * std::max<uint64_t>(tiles, 1)) +
           align_up(4 * std::max<uint64_t>(m, 1)) + align_up(4 * scan_sum_words(m)) + align_up(16);
}

// Exclusive scan of n u32 values in place (tile sums in `sums`, which must hold at least
// ceil(n / 4096) words); *total (device, nullable) receives the sum.
int scan_u32(cac_ctx *ctx, uint32_t *x, uint64_t n, uint32_t *sums, uint32_t *total) {
    cudaStream_t s = ctx->stream;
    const uint64_t nt = (n + kSTile - 1) / kSTile;
    if (nt == 0) {
        if (total) CAC_CUDA_TRY(cudaMemsetAsync(total, 0, 4, s));
        return CAC_OK;
    }
    scan_tile_sums<<<(unsigned)nt, kST, 0, s>>>(x, n, sums);
    scan_sums<<<1, 1024, 0, s>>>(sums, (uint32_t)nt, total);
    scan_apply<<<(unsigned)nt, kST, 0, s>>>(x, n, sums);
    CAC_CUDA_TRY(cudaGetLastError());
    return CAC_OK;
}

// The child edge list of labels lab (or the identity when lab is null) over k vertices: every
// non-loop edge (lab[a], lab[b], w) of the parent's m edges, sorted by (smaller, larger end) with
// equal pairs merged (u64 weight sums). Writes the pairs to oa/ob/ow (room for m entries) and the
// number of distinct pairs to *d_count (device). k * k must stay below 2^63.
template <typename WT>
int merge_edges(cac_ctx *ctx, const uint32_t *a, const uint32_t *b, const WT *w, uint64_t m, const uint32_t *lab,
                uint32_t k, uint32_t *oa, uint32_t *ob, uint64_t *ow, uint32_t *d_count, void *scratch) {
    cudaStream_t s = ctx->stream;
    if (m == 0) {
        CAC_CUDA_TRY(cudaMemsetAsync(d_count, 0, 4, s));
        return CAC_OK;
    }
    const uint64_t tiles = (m + kSTile - 1) / kSTile;
    if (tiles * kRadix > 0xFFFFFFFFull || m > 0xFFFFFFFFull) {
        set_error("merge_edges: too many edges for 32-bit offsets");
        return CAC_ERR_UNSUPPORTED;
    }
    char *p = static_cast<char *>(scratch);
    auto take = [&](size_t bytes) {
        char *q = p;
        p += align_up(bytes);
        return q;
    };
    uint64_t *k0 = reinterpret_cast<uint64_t *>(take(8 * m)), *v0 = reinterpret_cast<uint64_t *>(take(8 * m));
    uint64_t *k1 = reinterpret_cast<uint64_t *>(take(8 * m)), *v1 = reinterpret_cast<uint64_t *>(take(8 * m));
    uint32_t *hist = reinterpret_cast<uint32_t *>(take(4 * kRadix * tiles));
    uint32_t *slot = reinterpret_cast<uint32_t *>(take(4 * m));
    const uint64_t hn = kRadix * tiles;
    uint32_t *sums = reinterpret_cast<uint32_t *>(take(4 * scan_sum_words(m)));
    edge_keys<WT><<<grid_of(ctx, m), 256, 0, s>>>(a, b, w, m, lab, k, k0, v0);
    const uint64_t loop_key = (uint64_t)k * k;
    int bits = 1;
    while (bits < 64 && (loop_key >> bits) != 0) bits++;
    for (int shift = 0; shift < bits; shift += 8) {
        radix_hist<<<(unsigned)tiles, kST, 0, s>>>(k0, m, shift, hist, (uint32_t)tiles);
        CAC_TRY(scan_u32(ctx, hist, hn, sums, nullptr));
        radix_scatter<<<(unsigned)tiles, kST, 0, s>>>(k0, v0, m, shift, hist, (uint32_t)tiles, k1, v1);
        std::swap(k0, k1);
        std::swap(v0, v1);
    }
    seg_heads<<<grid_of(ctx, m), 256, 0, s>>>(k0, m, loop_key, slot);
    CAC_TRY(scan_u32(ctx, slot, m, sums, d_count));
    seg_merge<<<grid_of(ctx, m), 256, 0, s>>>(k0, v0, m, loop_key, k, slot, oa, ob,
                                              reinterpret_cast<unsigned long long *>(ow));
    CAC_CUDA_TRY(cudaGetLastError());
    return CAC_OK;
}

// The children of many tasks in one sort (see MergeTask): every task's merged pairs, task after
// task, each task's in sorted (smaller, larger end) order; counts[t] (device, zeroed here) gets task
// t's number of pairs, so task t's pairs start at the sum of the earlier counts. oa/ob/ow have room
// for the sum of the tasks' m. The tasks' in_off and key_off are filled in here.
int merge_edges_multi(cac_ctx *ctx, std::vector<MergeTask> &tasks, uint32_t *oa, uint32_t *ob, uint64_t *ow,
                      uint32_t *counts, void *scratch) {
    cudaStream_t s = ctx->stream;
    const uint32_t B = (uint32_t)tasks.size();
    if (B == 0) return CAC_OK;
    if (B > 65535) {
        set_error("merge_edges_multi: more than 65535 tasks in one call");
        return CAC_ERR_INVALID;
    }
    uint64_t M = 0, key_space = 0, mmax = 0;
    for (MergeTask &t : tasks) {
        t.in_off = M;
        t.key_off = key_space;
        M += t.m;
        key_space += (uint64_t)t.k * t.k;
        mmax = std::max(mmax, t.m);
    }
    CAC_CUDA_TRY(cudaMemsetAsync(counts, 0, 4ull * B, s));
    if (M == 0) return CAC_OK;
    const uint64_t tiles = (M + kSTile - 1) / kSTile;
    if (tiles * kRadix > 0xFFFFFFFFull || M > 0xFFFFFFFFull || key_space >= (1ull << 62)) {
        set_error("merge_edges_multi: too many edges for 32-bit offsets");
        return CAC_ERR_UNSUPPORTED;
    }
    char *p = static_cast<char *>(scratch);
    auto take = [&](size_t bytes) {
        char *q = p;
        p += align_up(bytes);
        return q;
    };
    uint64_t *k0 = reinterpret_cast<uint64_t *>(take(8 * M)), *v0 = reinterpret_cast<uint64_t *>(take(8 * M));
    uint64_t *k1 = reinterpret_cast<uint64_t *>(take(8 * M)), *v1 = reinterpret_cast<uint64_t *>(take(8 * M));
    uint32_t *hist = reinterpret_cast<uint32_t *>(take(4 * kRadix * tiles));
    uint32_t *slot = reinterpret_cast<uint32_t *>(take(4 * M));
    uint32_t *sums = reinterpret_cast<uint32_t *>(take(4 * scan_sum_words(M)));
    uint32_t *total = reinterpret_cast<uint32_t *>(take(16));
    MergeTask *dt = reinterpret_cast<MergeTask *>(take(sizeof(MergeTask) * B));
    CAC_CUDA_TRY(cudaMemcpyAsync(dt, tasks.data(), sizeof(MergeTask) * B, cudaMemcpyHostToDevice, s));
    const uint64_t hn = kRadix * tiles;
    const unsigned gx = (unsigned)std::max<uint64_t>(
        1, std::min<uint64_t>((mmax + 255) / 256, std::max<uint64_t>(1, (uint64_t)ctx->num_sms * 8 / B)));
    edge_keys_multi<<<dim3(gx, B), 256, 0, s>>>(dt, key_space, k0, v0);
    int bits = 1;
    while (bits < 64 && (key_space >> bits) != 0) bits++;
    for (int shift = 0; shift < bits; shift += 8) {
        radix_hist<<<(unsigned)tiles, kST, 0, s>>>(k0, M, shift, hist, (uint32_t)tiles);
        CAC_TRY(scan_u32(ctx, hist, hn, sums, nullptr));
        radix_scatter<<<(unsigned)tiles, kST, 0, s>>>(k0, v0, M, shift, hist, (uint32_t)tiles, k1, v1);
        std::swap(k0, k1);
        std::swap(v0, v1);
    }
    seg_heads<<<grid_of(ctx, M), 256, 0, s>>>(k0, M, key_space, slot);
    CAC_TRY(scan_u32(ctx, slot, M, sums, total));
    seg_merge_multi<<<grid_of(ctx, M), 256, 0, s>>>(k0, v0, M, key_space, dt, B, slot, oa, ob,
                                                    reinterpret_cast<unsigned long long *>(ow));
    task_counts<<<(B + 255) / 256, 256, 0, s>>>(k0, M, slot, total, dt, B, counts);
    CAC_CUDA_TRY(cudaGetLastError());
    return CAC_OK;
}

uint64_t merge_edges_multi_scratch(uint64_t M, uint32_t B) {
    return merge_edges_scratch(M) + align_up(16) + align_up(sizeof(MergeTask) * std::max<uint32_t>(B, 1));
}

template int merge_edges<uint32_t>(cac_ctx *, const uint32_t *, const uint32_t *, const uint32_t *, uint64_t,
                                   const uint32_t *, uint32_t, uint32_t *, uint32_t *, uint64_t *, uint32_t *, void *);
template int merge_edges<uint64_t>(cac_ctx *, const uint32_t *, const uint32_t *, const uint64_t *, uint64_t,
                                   const uint32_t *, uint32_t, uint32_t *, uint32_t *, uint64_t *, uint32_t *, void *);

}  // namespace cac
