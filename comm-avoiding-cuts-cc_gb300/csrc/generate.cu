// Seeded synthetic graphs generated on the device, edge for edge identical to the host generators
// in graphgen.py (same splitmix64 counter hashing, same edge order, same weights).
//
// The reference builds its inputs with external generators (utils/generate.py:10-32 over
// NetworkX, input_generators/rmat_driver.sh:13-16 over PaRMAT, src/executables/er_generator.cpp
// and sw_generator.cpp) and writes them to edge-list files. Here a generated graph is made
// straight in HBM: R-MAT scale 22 (67M edges) takes milliseconds instead of a minute of host
// work plus a file.
//
// hash(seed, stream, i) = mix(i * 0x9E3779B97F4A7C15 + mix(seed * 0x100000001B3 + stream * 0x9E3779B1))
// with mix the splitmix64 finaliser; a uniform integer in [lo, hi] is lo + ((hash >> 32) * span >> 32).
// Families whose edges are kept by a test (G(n, p), G(n, M) without self-loops) are compacted in
// index order: a count pass per tile of 1024 candidates, an exclusive scan of the tile counts on
// the host, and a write pass that ranks the kept candidates inside each tile with a block scan.
#include "cac_internal.h"

#include <cmath>
#include <vector>

namespace cac {
namespace {

constexpr int kGT = 256;                // threads per generator block
constexpr int kPer = 4;                 // candidates per thread
constexpr int kTile = kGT * kPer;       // candidates per block
constexpr uint64_t kGold = 0x9E3779B97F4A7C15ull;

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z ^= z >> 30;
    z *= 0xBF58476D1CE4E5B9ull;
    z ^= z >> 27;
    z *= 0x94D049BB133111EBull;
    z ^= z >> 31;
    return z;
}

uint64_t stream_base(uint64_t seed, uint64_t stream) { return mix64(seed * 0x100000001B3ull + stream * 0x9E3779B1ull); }

__device__ __forceinline__ uint64_t h64(uint64_t base, uint64_t i) { return mix64(i * kGold + base); }

__device__ __forceinline__ uint32_t uni(uint64_t base, uint64_t i, uint32_t lo, uint32_t hi) {
    const uint64_t span = (uint64_t)hi - lo + 1;
    return lo + (uint32_t)(((h64(base, i) >> 32) * span) >> 32);
}

// p * 2^64 truncated, saturated at 2^64 - 1 (the host generator's threshold)
uint64_t threshold(double p) {
    const double x = p * 18446744073709551616.0;
    if (!(x > 0.0)) return 0;
    if (x >= 18446744073709551616.0) return ~0ull;
    return (uint64_t)x;
}

struct Weights {
    uint64_t base;  // stream 7
    uint32_t lo, hi;
    uint32_t ones;  // unweighted: every weight 1
};

__device__ __forceinline__ uint32_t weight_of(const Weights &w, uint64_t e) {
    return w.ones ? 1u : uni(w.base, e, w.lo, w.hi);
}

template <int NT>
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t x, uint32_t &total) {
    __shared__ uint32_t warp_sums[NT / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t inc = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) warp_sums[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        uint32_t s = lane < NT / 32 ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < NT / 32) warp_sums[lane] = s;
    }
    __syncthreads();
    total = warp_sums[NT / 32 - 1];
    const uint32_t off = wid ? warp_sums[wid - 1] : 0;
    __syncthreads();
    return off + inc - x;
}

// ---- G(n, p): candidates are the pairs i < j in row-major order, hashed at i * n + j (stream 1)

struct PairSpace {
    uint32_t n;
    uint64_t total;  // n (n - 1) / 2
};

// first pair position of row i
__device__ __forceinline__ uint64_t row_start(uint64_t n, uint64_t i) { return i * (n - 1) - i * (i - 1) / 2; }

__device__ __forceinline__ void pair_at(const PairSpace &P, uint64_t pos, uint32_t &i, uint32_t &j) {
    uint64_t lo = 0, hi = P.n - 2;  // last row whose start <= pos
    while (lo < hi) {
        const uint64_t mid = (lo + hi + 1) >> 1;
        if (row_start(P.n, mid) <= pos) lo = mid; else hi = mid - 1;
    }
    i = (uint32_t)lo;
    j = (uint32_t)(lo + 1 + (pos - row_start(P.n, lo)));
}

struct GnpArgs {
    PairSpace P;
    uint64_t base, thr;
};

// keeps of thread t's kPer consecutive candidates, as a bit mask, with their first pair
__device__ __forceinline__ uint32_t gnp_mask(const GnpArgs &A, uint64_t first, uint32_t &i0, uint32_t &j0) {
    uint32_t mask = 0;
    if (first >= A.P.total) return 0;
    pair_at(A.P, first, i0, j0);
    uint32_t i = i0, j = j0;
    for (int k = 0; k < kPer && first + k < A.P.total; k++) {
        if (h64(A.base, (uint64_t)i * A.P.n + j) < A.thr) mask |= 1u << k;
        if (++j == A.P.n) {
            i++;
            j = i + 1;
        }
    }
    return mask;
}

__global__ void __launch_bounds__(kGT) gnp_count(GnpArgs A, uint32_t *tile_count) {
    const uint64_t first = ((uint64_t)blockIdx.x * kGT + threadIdx.x) * kPer;
    uint32_t i0, j0;
    uint32_t c = __popc(gnp_mask(A, first, i0, j0));
    uint32_t tot;
    block_excl_scan<kGT>(c, tot);
    if (threadIdx.x == 0) tile_count[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kGT) gnp_write(GnpArgs A, const uint64_t *tile_off, uint32_t *U, uint32_t *V) {
    const uint64_t first = ((uint64_t)blockIdx.x * kGT + threadIdx.x) * kPer;
    uint32_t i0 = 0, j0 = 0;
    const uint32_t mask = gnp_mask(A, first, i0, j0);
    uint32_t tot;
    uint64_t out = tile_off[blockIdx.x] + block_excl_scan<kGT>(__popc(mask), tot);
    uint32_t i = i0, j = j0;
    for (int k = 0; k < kPer; k++) {
        if (mask >> k & 1u) {
            U[out] = i;
            V[out] = j;
            out++;
        }
        if (++j == A.P.n) {
            i++;
            j = i + 1;
        }
    }
}

// ---- G(n, M): candidate e draws u (stream 2) and v (stream 3); a self-loop redraws v once
// (stream 4) and is dropped if it persists

struct GnmArgs {
    uint64_t m0;
    uint32_t n;
    uint64_t b2, b3, b4;
};

__device__ __forceinline__ bool gnm_edge(const GnmArgs &A, uint64_t e, uint32_t &u, uint32_t &v) {
    u = uni(A.b2, e, 0, A.n - 1);
    v = uni(A.b3, e, 0, A.n - 1);
    if (u == v) v = uni(A.b4, e, 0, A.n - 1);
    return u != v;
}

__global__ void __launch_bounds__(kGT) gnm_count(GnmArgs A, uint32_t *tile_count) {
    const uint64_t first = ((uint64_t)blockIdx.x * kGT + threadIdx.x) * kPer;
    uint32_t c = 0, u, v;
    for (int k = 0; k < kPer; k++)
        if (first + k < A.m0 && gnm_edge(A, first + k, u, v)) c++;
    uint32_t tot;
    block_excl_scan<kGT>(c, tot);
    if (threadIdx.x == 0) tile_count[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kGT) gnm_write(GnmArgs A, const uint64_t *tile_off, uint32_t *U, uint32_t *V) {
    const uint64_t first = ((uint64_t)blockIdx.x * kGT + threadIdx.x) * kPer;
    uint32_t us[kPer], vs[kPer], c = 0;
    for (int k = 0; k < kPer; k++)
        if (first + k < A.m0 && gnm_edge(A, first + k, us[c], vs[c])) c++;
    uint32_t tot;
    uint64_t out = tile_off[blockIdx.x] + block_excl_scan<kGT>(c, tot);
    for (uint32_t k = 0; k < c; k++) {
        U[out + k] = us[k];
        V[out + k] = vs[k];
    }
}

// ---- fixed-size families: one thread per edge

struct WsArgs {
    uint32_t n, half;
    uint64_t m;
    uint64_t b11, b12, thr;
};

__global__ void ws_kernel(WsArgs A, uint32_t *U, uint32_t *V) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < A.m; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = e / A.half, j = e % A.half + 1;
        const uint32_t u = (uint32_t)i;
        uint32_t v = (uint32_t)((i + j) % A.n);
        const bool rew = h64(A.b11, e) < A.thr;
        const uint32_t x = uni(A.b12, e, 0, A.n - 1);
        if (rew && x != u) v = x;
        U[e] = u;
        V[e] = v;
    }
}

struct RmatArgs {
    uint32_t scale;
    uint64_t m;
    uint64_t ta, tb, tc;
    uint64_t base[32];  // streams 100 + level
};

__global__ void rmat_kernel(const RmatArgs A, uint32_t *U, uint32_t *V) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < A.m; e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t u = 0, v = 0;
        for (uint32_t l = 0; l < A.scale; l++) {
            const uint64_t h = h64(A.base[l], e);
            const uint32_t bu = h >= A.tb ? 1u : 0u;
            const uint32_t bv = ((h >= A.ta && h < A.tb) || h >= A.tc) ? 1u : 0u;
            u = (u << 1) | bu;
            v = (v << 1) | bv;
        }
        U[e] = u;
        V[e] = v;
    }
}

__global__ void complete_kernel(PairSpace P, uint32_t *U, uint32_t *V) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < P.total; e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t i, j;
        pair_at(P, e, i, j);
        U[e] = i;
        V[e] = j;
    }
}

__global__ void weights_kernel(Weights w, uint64_t m, uint32_t *W) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x)
        W[e] = weight_of(w, e);
}

unsigned grid_for(const cac_ctx *ctx, uint64_t work) {
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((work + 255) / 256, (uint64_t)ctx->num_sms * 16));
}

// Edge buffers of a generated graph before it is handed to graph_create (which validates it).
struct EdgeBufs {
    cac_ctx *ctx;
    void *p = nullptr;
    size_t bytes = 0;
    uint32_t *U = nullptr, *V = nullptr, *W = nullptr;
    explicit EdgeBufs(cac_ctx *c) : ctx(c) {}
    ~EdgeBufs() {
        if (p) {
            cudaStreamSynchronize(ctx->stream);
            dev_free(ctx, p, bytes);
        }
    }
    int alloc(uint64_t m) {
        const size_t b = align_up(std::max<uint64_t>(m, 1) * 4);
        bytes = 3 * b;
        CAC_TRY(dev_alloc(ctx, &p, bytes));
        U = static_cast<uint32_t *>(p);
        V = reinterpret_cast<uint32_t *>(static_cast<char *>(p) + b);
        W = reinterpret_cast<uint32_t *>(static_cast<char *>(p) + 2 * b);
        return CAC_OK;
    }
};

// Tile counts -> exclusive offsets (host scan); returns the number of kept candidates.
int scan_tiles(cac_ctx *ctx, const uint32_t *d_count, uint64_t tiles, uint64_t *d_off, uint64_t *kept) {
    std::vector<uint32_t> c(tiles);
    std::vector<uint64_t> off(tiles);
    CAC_CUDA_TRY(cudaMemcpyAsync(c.data(), d_count, tiles * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CAC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    uint64_t acc = 0;
    for (uint64_t t = 0; t < tiles; t++) {
        off[t] = acc;
        acc += c[t];
    }
    CAC_CUDA_TRY(cudaMemcpyAsync(d_off, off.data(), tiles * 8, cudaMemcpyHostToDevice, ctx->stream));
    CAC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    *kept = acc;
    return CAC_OK;
}

int generate(cac_ctx *ctx, const cac_gen_spec &S, cac_graph **out) {
    cudaStream_t s = ctx->stream;
    const uint64_t seed = S.seed;
    Weights wt{stream_base(seed, 7), S.wmin, S.wmax, 0};
    EdgeBufs eb(ctx);
    uint32_t n = S.n;
    uint64_t m = 0;
    switch (S.family) {
    case CAC_GEN_ERDOS_RENYI: {
        if (S.n < 2 || !(S.p >= 0.0 && S.p <= 1.0)) break;
        GnpArgs A{PairSpace{S.n, (uint64_t)S.n * (S.n - 1) / 2}, stream_base(seed, 1), threshold(S.p)};
        const uint64_t tiles = (A.P.total + kTile - 1) / kTile;
        void *cnt = nullptr, *off = nullptr;
        CAC_TRY(dev_alloc(ctx, &cnt, tiles * 4));
        int st = dev_alloc(ctx, &off, tiles * 8);
        if (st == CAC_OK) {
            gnp_count<<<(unsigned)tiles, kGT, 0, s>>>(A, static_cast<uint32_t *>(cnt));
            st = scan_tiles(ctx, static_cast<uint32_t *>(cnt), tiles, static_cast<uint64_t *>(off), &m);
        }
        if (st == CAC_OK && m > 0xFFFFFFFFull) {
            set_error("generated graph has more than 2^32-1 edges");
            st = CAC_ERR_UNSUPPORTED;
        }
        if (st == CAC_OK) st = eb.alloc(m);
        if (st == CAC_OK && m) gnp_write<<<(unsigned)tiles, kGT, 0, s>>>(A, static_cast<uint64_t *>(off), eb.U, eb.V);
        cudaStreamSynchronize(s);
        if (off) dev_free(ctx, off, tiles * 8);
        dev_free(ctx, cnt, tiles * 4);
        CAC_TRY(st);
        wt.ones = S.wmax > 1 ? 0u : 1u;
        break;
    }
    case CAC_GEN_ERDOS_RENYI_M: {
        if (S.n < 1 || !(S.avg_degree >= 0.0)) break;
        GnmArgs A{(uint64_t)std::floor((double)S.n * S.avg_degree / 2.0), S.n, stream_base(seed, 2),
                  stream_base(seed, 3), stream_base(seed, 4)};
        if (A.m0 > 0xFFFFFFFFull) {
            set_error("generated graph has more than 2^32-1 edges");
            return CAC_ERR_UNSUPPORTED;
        }
        const uint64_t tiles = std::max<uint64_t>(1, (A.m0 + kTile - 1) / kTile);
        void *cnt = nullptr, *off = nullptr;
        CAC_TRY(dev_alloc(ctx, &cnt, tiles * 4));
        int st = dev_alloc(ctx, &off, tiles * 8);
        if (st == CAC_OK) {
            gnm_count<<<(unsigned)tiles, kGT, 0, s>>>(A, static_cast<uint32_t *>(cnt));
            st = scan_tiles(ctx, static_cast<uint32_t *>(cnt), tiles, static_cast<uint64_t *>(off), &m);
        }
        if (st == CAC_OK) st = eb.alloc(m);
        if (st == CAC_OK && m) gnm_write<<<(unsigned)tiles, kGT, 0, s>>>(A, static_cast<uint64_t *>(off), eb.U, eb.V);
        cudaStreamSynchronize(s);
        if (off) dev_free(ctx, off, tiles * 8);
        dev_free(ctx, cnt, tiles * 4);
        CAC_TRY(st);
        break;
    }
    case CAC_GEN_WATTS_STROGATZ: {
        if (S.n < 1 || S.k < 2 || (S.k & 1) || S.k >= S.n || !(S.p >= 0.0 && S.p <= 1.0)) break;
        WsArgs A{S.n, S.k / 2, (uint64_t)S.n * (S.k / 2), stream_base(seed, 11), stream_base(seed, 12), threshold(S.p)};
        m = A.m;
        CAC_TRY(eb.alloc(m));
        ws_kernel<<<grid_for(ctx, m), 256, 0, s>>>(A, eb.U, eb.V);
        break;
    }
    case CAC_GEN_RMAT: {
        const double d = 1.0 - S.a - S.b - S.c;
        if (S.scale < 1 || S.scale > 31 || S.edge_factor == 0 || !(S.a >= 0 && S.b >= 0 && S.c >= 0 && d >= 0)) break;
        RmatArgs A{};
        A.scale = S.scale;
        n = 1u << S.scale;
        A.m = (uint64_t)S.edge_factor * n;
        if (A.m > 0xFFFFFFFFull) {
            set_error("generated graph has more than 2^32-1 edges");
            return CAC_ERR_UNSUPPORTED;
        }
        A.ta = threshold(S.a);
        A.tb = threshold(S.a + S.b);
        A.tc = threshold(S.a + S.b + S.c);
        for (uint32_t l = 0; l < S.scale; l++) A.base[l] = stream_base(seed, 100 + l);
        m = A.m;
        CAC_TRY(eb.alloc(m));
        rmat_kernel<<<grid_for(ctx, m), 256, 0, s>>>(A, eb.U, eb.V);
        wt.ones = S.wmax > 1 ? 0u : 1u;
        break;
    }
    case CAC_GEN_COMPLETE: {
        if (S.n < 2) break;
        PairSpace P{S.n, (uint64_t)S.n * (S.n - 1) / 2};
        m = P.total;
        if (m > 0xFFFFFFFFull) {
            set_error("generated graph has more than 2^32-1 edges");
            return CAC_ERR_UNSUPPORTED;
        }
        CAC_TRY(eb.alloc(m));
        complete_kernel<<<grid_for(ctx, m), 256, 0, s>>>(P, eb.U, eb.V);
        break;
    }
    default:
        break;
    }
    if (!eb.p) {
        set_error("cac_graph_generate: unknown family or parameters out of range");
        return CAC_ERR_INVALID;
    }
    if (m) weights_kernel<<<grid_for(ctx, m), 256, 0, s>>>(wt, m, eb.W);
    CAC_CUDA_TRY(cudaGetLastError());
    return graph_create(ctx, n, m, eb.U, eb.V, eb.W, CAC_DEVICE, out);
}

}  // namespace
}  // namespace cac

using namespace cac;

extern "C" int cac_graph_generate(cac_ctx *ctx, const cac_gen_spec *spec, cac_graph **out) {
    if (!ctx || !spec || !out) {
        set_error("cac_graph_generate: invalid argument");
        return CAC_ERR_INVALID;
    }
    *out = nullptr;
    CAC_CUDA_TRY(cudaSetDevice(ctx->device));
    if (spec->wmin == 0 || spec->wmax < spec->wmin) {
        set_error("cac_graph_generate: weights need 1 <= wmin <= wmax");
        return CAC_ERR_INVALID;
    }
    return generate(ctx, *spec, out);
}
