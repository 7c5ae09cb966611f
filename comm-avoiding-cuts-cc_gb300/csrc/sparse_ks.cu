// Sparse Karger-Stein nodes: the part of a trial above the dense limit, or on graphs with fewer
// than N^2 / 32 edges. The reference switches to its sparse recursion there
// (src/karger-stein/co_mincut.h:401-405): every node keeps an edge list, each child contracts a
// copy by exponential edge scores and a prefix connected components (co_mincut.h:74-155,
// sparse_graph.hpp:614-672), then relabels and compacts (sparse_graph.hpp:451-545). Here:
//   children      both children of every sparse node of a level are contracted together by the
//                 Stage 1 rounds of shrink_big.cu (weighted draws over the edges that are not
//                 loops, contracted in draw order, keys (k0, trial, 1 + child heap index, 0)):
//                 one grid over all tasks, each task on its own edge list
//   relabel/merge the child's edges relabelled by rank-of-minimum labels, sorted by (smaller,
//                 larger end) with the device radix sort and merged with u64 weight sums
//                 (sort.cu): the reference's WeightedIteratedSparseSampling::reduce step
//   hand-over     a child that is dense by the shared rule becomes its matrix (one store per
//                 merged pair and direction) and joins the level-synchronous dense engine; the
//                 others are the next sparse level
//   roots         a sparse root also delivers its minimum weighted degree; a node without edges
//                 has cut 0
// Every size is read back between the steps of a level (a sparse level is a few large tasks, not
// a latency-bound stream of small ones). Trial values equal the oracle's replay (oracle/mincut.c).
#include "cac_internal.h"

#include <algorithm>
#include <map>
#include <vector>

namespace cac {
namespace {

// One dense child of a chunk: its merged pairs (slices of the chunk's list buffer) and its matrix.
struct DenseFromPairs {
    const uint32_t *a, *b;
    const uint64_t *w;
    uint64_t m, ld;
    void *mat;
};

template <typename WT>
__global__ void sparse_degree(const uint32_t *a, const uint32_t *b, const WT *w, uint64_t m, unsigned long long *deg) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t x = a[e], y = b[e];
        if (x == y) continue;
        atomicAdd(deg + x, (unsigned long long)w[e]);
        atomicAdd(deg + y, (unsigned long long)w[e]);
    }
}

__global__ void sparse_min(const unsigned long long *deg, uint32_t n, unsigned long long *out) {
    unsigned long long x = ~0ull;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        x = min(x, deg[i]);
    for (int o = 16; o > 0; o >>= 1) x = min(x, __shfl_xor_sync(0xffffffffu, x, o));
    if ((threadIdx.x & 31) == 0) atomicMin(out, x);
}

// cut[i] = min(cut[i], *value) for a list of trial cuts (value null: 0)
__global__ void cuts_min(unsigned long long *const *cuts, uint32_t count, const unsigned long long *value) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        atomicMin(cuts[i], value ? *value : 0ull);
}

// The dense matrix of a merged edge list (each pair once): both directions stored; CTA row y of
// the grid serves child y.
template <typename Tm>
__global__ void dense_from_pairs(const DenseFromPairs *__restrict__ d) {
    const DenseFromPairs c = d[blockIdx.y];
    Tm *mat = static_cast<Tm *>(c.mat);
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < c.m; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t x = c.a[e], y = c.b[e];
        mat[x * c.ld + y] = (Tm)c.w[e];
        mat[y * c.ld + x] = (Tm)c.w[e];
    }
}

// The dense children of a chunk, one launch per entry width (descs: room for both lists).
int dense_children(cac_ctx *ctx, const std::vector<DenseFromPairs> &d32, const std::vector<DenseFromPairs> &d64,
                   DenseFromPairs *descs) {
    cudaStream_t s = ctx->stream;
    const std::vector<DenseFromPairs> *lists[2] = {&d32, &d64};
    DenseFromPairs *at = descs;
    for (int wi = 0; wi < 2; wi++) {
        const std::vector<DenseFromPairs> &v = *lists[wi];
        for (size_t i0 = 0; i0 < v.size(); i0 += 65535) {
            const size_t n = std::min<size_t>(65535, v.size() - i0);
            uint64_t mmax = 1;
            for (size_t i = i0; i < i0 + n; i++) mmax = std::max(mmax, v[i].m);
            CAC_CUDA_TRY(cudaMemcpyAsync(at, v.data() + i0, sizeof(DenseFromPairs) * n, cudaMemcpyHostToDevice, s));
            const dim3 grid((unsigned)std::max<uint64_t>(
                                1, std::min<uint64_t>((mmax + 255) / 256, std::max<uint64_t>(1, (uint64_t)ctx->num_sms * 8 / n))),
                            (unsigned)n);
            if (wi == 0) dense_from_pairs<uint32_t><<<grid, 256, 0, s>>>(at);
            else dense_from_pairs<uint64_t><<<grid, 256, 0, s>>>(at);
            CAC_CUDA_TRY(cudaGetLastError());
            at += n;
        }
    }
    return CAC_OK;
}

unsigned grid_of(cac_ctx *ctx, uint64_t work) {
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((work + 255) / 256, (uint64_t)ctx->num_sms * 8));
}

uint64_t ld_of(uint32_t N) { return ((uint64_t)N + 3) & ~(uint64_t)3; }

// A stream-ordered temporary from the ctx pool, freed when it goes out of scope.
struct Temp {
    cac_ctx *ctx;
    void *p = nullptr;
    size_t bytes = 0;
    explicit Temp(cac_ctx *c) : ctx(c) {}
    ~Temp() { if (p) stream_free(ctx, p, bytes); }
    int get(size_t b) {
        if (b <= bytes) return CAC_OK;
        if (p) stream_free(ctx, p, bytes);
        p = nullptr;
        bytes = 0;
        CAC_TRY(stream_alloc(ctx, &p, std::max<size_t>(b, 256)));
        bytes = std::max<size_t>(b, 256);
        return CAC_OK;
    }
    template <typename T> T *as() const { return static_cast<T *>(p); }
};

// Minimum weighted degree of every distinct root graph, min'd into its trials' cuts.
int root_bounds(cac_ctx *ctx, const std::vector<SparseNode> &nodes) {
    cudaStream_t s = ctx->stream;
    std::map<const uint32_t *, std::vector<uint64_t *>> by_graph;
    std::map<const uint32_t *, const SparseNode *> first;
    for (const SparseNode &nd : nodes) {
        if (!nd.is_root || nd.m == 0) continue;
        by_graph[nd.a].push_back(nd.cut);
        first.emplace(nd.a, &nd);
    }
    for (auto &kv : by_graph) {
        const SparseNode &nd = *first[kv.first];
        Temp deg(ctx), cuts(ctx);
        CAC_TRY(deg.get(((size_t)nd.N + 1) * 8));
        CAC_TRY(cuts.get(kv.second.size() * sizeof(uint64_t *)));
        unsigned long long *d = deg.as<unsigned long long>(), *res = d + nd.N;
        CAC_CUDA_TRY(cudaMemsetAsync(d, 0, (size_t)nd.N * 8, s));
        CAC_CUDA_TRY(cudaMemsetAsync(res, 0xFF, 8, s));
        if (nd.w64)
            sparse_degree<uint64_t><<<grid_of(ctx, nd.m), 256, 0, s>>>(nd.a, nd.b, static_cast<const uint64_t *>(nd.w),
                                                                       nd.m, d);
        else
            sparse_degree<uint32_t><<<grid_of(ctx, nd.m), 256, 0, s>>>(nd.a, nd.b, static_cast<const uint32_t *>(nd.w),
                                                                       nd.m, d);
        sparse_min<<<grid_of(ctx, nd.N), 256, 0, s>>>(d, nd.N, res);
        CAC_CUDA_TRY(cudaMemcpyAsync(cuts.p, kv.second.data(), kv.second.size() * sizeof(uint64_t *),
                                     cudaMemcpyHostToDevice, s));
        cuts_min<<<grid_of(ctx, kv.second.size()), 256, 0, s>>>(cuts.as<unsigned long long *>(),
                                                                (uint32_t)kv.second.size(), res);
        CAC_CUDA_TRY(cudaGetLastError());
        CAC_CUDA_TRY(cudaStreamSynchronize(s));  // the host pointer list and the temporaries go out of scope
    }
    return CAC_OK;
}

int zero_cuts(cac_ctx *ctx, const std::vector<uint64_t *> &cuts) {
    if (cuts.empty()) return CAC_OK;
    cudaStream_t s = ctx->stream;
    Temp d(ctx);
    CAC_TRY(d.get(cuts.size() * sizeof(uint64_t *)));
    CAC_CUDA_TRY(cudaMemcpyAsync(d.p, cuts.data(), cuts.size() * sizeof(uint64_t *), cudaMemcpyHostToDevice, s));
    cuts_min<<<grid_of(ctx, cuts.size()), 256, 0, s>>>(d.as<unsigned long long *>(), (uint32_t)cuts.size(), nullptr);
    CAC_CUDA_TRY(cudaGetLastError());
    CAC_CUDA_TRY(cudaStreamSynchronize(s));
    return CAC_OK;
}

}  // namespace

int sparse_phase(cac_ctx *ctx, KsEngine &eng, std::vector<SparseNode> nodes) {
    cudaStream_t s = ctx->stream;
    int st = CAC_OK;
    auto release_all = [&](std::vector<SparseNode> &v) {
        for (SparseNode &nd : v)
            if (nd.buf) eng.release(nd.buf);
        v.clear();
    };
    // a chunk of children: contraction scratch within 4 GB and at most kChunkEdges parent edges (the
    // sort of one chunk takes 40 bytes per parent edge, its merged lists 16)
    constexpr uint64_t kChunkEdges = 64ull << 20;
    while (!nodes.empty()) {
        st = root_bounds(ctx, nodes);
        // the children of every node with edges: two contraction tasks each
        struct Child {
            const SparseNode *src;
            uint64_t h;
            uint32_t target;
        };
        std::vector<Child> children;
        std::vector<uint64_t *> zero;
        for (const SparseNode &nd : nodes) {
            if (nd.m == 0) {
                zero.push_back(nd.cut);  // no edge between its vertices: cut 0
                continue;
            }
            const uint32_t target = (uint32_t)ks_target((int)nd.N);
            for (uint64_t c = 0; c < 2; c++) children.push_back(Child{&nd, 2 * nd.h + c, target});
        }
        if (st == CAC_OK) st = zero_cuts(ctx, zero);
        std::vector<SparseNode> next;
        size_t c0 = 0;
        while (st == CAC_OK && c0 < children.size()) {
            size_t c1 = c0;
            uint64_t bytes = 0, labw = 0, M = 0;
            while (c1 < children.size() && c1 - c0 < 65535) {
                const SparseNode &nd = *children[c1].src;
                const uint64_t b = shrink_task_scratch(nd.N, nd.m) + align_up(4ull * nd.N);
                if (c1 > c0 && (bytes + b > (4ull << 30) || M + nd.m > kChunkEdges)) break;
                bytes += b;
                labw += nd.N;
                M += nd.m;
                c1++;
            }
            const uint32_t B = (uint32_t)(c1 - c0);
            Temp lab(ctx), kout(ctx), scr(ctx), merge_scr(ctx), counts(ctx);
            if ((st = lab.get(labw * 4)) != CAC_OK || (st = kout.get(B * 4)) != CAC_OK ||
                (st = counts.get(B * 4)) != CAC_OK || (st = merge_scr.get(merge_edges_multi_scratch(M, B))) != CAC_OK)
                break;
            // 1. contract every child's copy of its parent (Stage 1 rounds, all tasks together)
            std::vector<ShrinkTask> tasks;
            uint64_t lo = 0;
            for (size_t i = c0; i < c1; i++) {
                const SparseNode &nd = *children[i].src;
                tasks.push_back(ShrinkTask{nd.a, nd.b, nd.w, nd.w64, nd.m, nd.N, children[i].target, nd.k0, nd.idx,
                                           1 + children[i].h, lab.as<uint32_t>() + lo,
                                           kout.as<uint32_t>() + (i - c0), 0});
                lo += nd.N;
            }
            if ((st = scr.get(shrink_tasks_scratch(tasks))) != CAC_OK) break;
            if ((st = shrink_tasks(ctx, tasks, scr.p)) != CAC_OK) break;
            std::vector<uint32_t> kk(B), mm(B);
            if (cudaMemcpyAsync(kk.data(), kout.p, B * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess) {
                set_error("sparse Karger-Stein: reading the contracted sizes failed");
                st = CAC_ERR_CUDA;
                break;
            }
            // 2. relabel, sort and merge every child's edges in one sort; the lists share one buffer
            std::vector<MergeTask> mt(B);
            lo = 0;
            for (uint32_t b = 0; b < B; b++) {
                const SparseNode &nd = *children[c0 + b].src;
                mt[b] = MergeTask{nd.a, nd.b, nd.w, nd.w64 ? 1u : 0u, kk[b], nd.m, lab.as<uint32_t>() + lo, 0, 0};
                lo += nd.N;
            }
            const uint64_t cap = std::max<uint64_t>(M, 1);
            MatBuf *lists = nullptr;
            if ((st = eng.alloc(align_up(cap * 4) * 2 + align_up(cap * 8), &lists)) != CAC_OK) break;
            lists->refs++;  // this scope's reference
            char *p = static_cast<char *>(lists->p);
            uint32_t *oa = reinterpret_cast<uint32_t *>(p), *ob = reinterpret_cast<uint32_t *>(p + align_up(cap * 4));
            uint64_t *ow = reinterpret_cast<uint64_t *>(p + 2 * align_up(cap * 4));
            st = merge_edges_multi(ctx, mt, oa, ob, ow, counts.as<uint32_t>(), merge_scr.p);
            if (st == CAC_OK && (cudaMemcpyAsync(mm.data(), counts.p, B * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                                 cudaStreamSynchronize(s) != cudaSuccess)) {
                set_error("sparse Karger-Stein: reading the merged edge counts failed");
                st = CAC_ERR_CUDA;
            }
            // 3. place every child: cut 0 without edges, a dense matrix, or the next sparse level
            std::vector<uint64_t> start(B + 1, 0);
            for (uint32_t b = 0; b < B; b++) start[b + 1] = start[b] + mm[b];
            std::vector<uint64_t *> zcut;
            std::vector<DenseFromPairs> dense32, dense64;
            uint64_t dense_bytes = 0;
            std::vector<uint64_t> mat_off(B, 0);
            for (uint32_t b = 0; b < B && st == CAC_OK; b++) {
                const SparseNode &nd = *children[c0 + b].src;
                const uint32_t k = kk[b];
                if (mm[b] == 0 || k < 2) {
                    zcut.push_back(nd.cut);
                } else if (ks_is_dense(ctx, k, mm[b])) {
                    mat_off[b] = dense_bytes;
                    dense_bytes += align_up(k * ld_of(k) * (nd.small ? 4 : 8));
                }
            }
            MatBuf *mats = nullptr;
            if (st == CAC_OK && dense_bytes) {
                st = eng.alloc(dense_bytes, &mats);
                if (st == CAC_OK) {
                    mats->refs++;  // this scope's reference
                    if (cudaMemsetAsync(mats->p, 0, dense_bytes, s) != cudaSuccess) {
                        set_error("sparse Karger-Stein: clearing the dense children failed");
                        st = CAC_ERR_CUDA;
                    }
                }
            }
            if (st == CAC_OK) st = zero_cuts(ctx, zcut);
            for (uint32_t b = 0; b < B && st == CAC_OK; b++) {
                const SparseNode &nd = *children[c0 + b].src;
                const uint32_t k = kk[b];
                if (mm[b] == 0 || k < 2) continue;
                const uint64_t first = start[b];
                if (ks_is_dense(ctx, k, mm[b])) {
                    unsigned char *mat = static_cast<unsigned char *>(mats->p) + mat_off[b];
                    (nd.small ? dense32 : dense64)
                        .push_back(DenseFromPairs{oa + first, ob + first, ow + first, mm[b], ld_of(k), mat});
                    eng.add(KNode{nd.cut, nd.k0, nd.idx, children[c0 + b].h, k, 0, nd.small, nd.query, mat, mats});
                } else {
                    lists->refs++;  // the next level's node holds the shared list buffer
                    next.push_back(SparseNode{nd.cut, nd.k0, nd.idx, children[c0 + b].h, k, mm[b], oa + first,
                                              ob + first, ow + first, true, false, nd.small, nd.query, lists});
                }
            }
            Temp descs(ctx);
            if (st == CAC_OK && (!dense32.empty() || !dense64.empty())) {
                st = descs.get(sizeof(DenseFromPairs) * (dense32.size() + dense64.size()));
                if (st == CAC_OK) st = dense_children(ctx, dense32, dense64, descs.as<DenseFromPairs>());
            }
            if (mats) eng.release(mats);
            eng.release(lists);
            if (st == CAC_OK) {
                const cudaError_t e = cudaStreamSynchronize(s);  // temporaries go out of scope
                if (e != cudaSuccess) {
                    set_error(std::string("sparse Karger-Stein: ") + cudaGetErrorString(e));
                    st = CAC_ERR_CUDA;
                }
            }
            c0 = c1;
        }
        release_all(nodes);
        if (st != CAC_OK) {
            release_all(next);
            return st;
        }
        nodes.swap(next);
    }
    return CAC_OK;
}

}  // namespace cac
