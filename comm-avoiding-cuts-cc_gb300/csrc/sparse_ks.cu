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

// The dense matrix of a merged edge list (each pair once): both directions stored.
template <typename Tm>
__global__ void dense_from_pairs(const uint32_t *a, const uint32_t *b, const uint64_t *w, uint64_t m, uint64_t ld,
                                 Tm *mat) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t x = a[e], y = b[e];
        mat[x * ld + y] = (Tm)w[e];
        mat[y * ld + x] = (Tm)w[e];
    }
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
            // a chunk of tasks whose contraction scratch and labels stay within 4 GB
            size_t c1 = c0;
            uint64_t bytes = 0, labw = 0, mmax = 1;
            std::vector<ShrinkTask> tasks;
            while (c1 < children.size() && c1 - c0 < 65535) {
                const SparseNode &nd = *children[c1].src;
                const uint64_t b = shrink_task_scratch(nd.N, nd.m) + align_up(4ull * nd.N);
                if (c1 > c0 && bytes + b > (4ull << 30)) break;
                bytes += b;
                labw += nd.N;
                mmax = std::max<uint64_t>(mmax, nd.m);
                c1++;
            }
            const uint32_t B = (uint32_t)(c1 - c0);
            Temp lab(ctx), kout(ctx), scr(ctx), merge_scr(ctx), counts(ctx);
            if ((st = lab.get(labw * 4)) != CAC_OK || (st = kout.get(B * 4)) != CAC_OK ||
                (st = counts.get(B * 4)) != CAC_OK || (st = merge_scr.get(merge_edges_scratch(mmax))) != CAC_OK)
                break;
            uint64_t lo = 0;
            for (size_t i = c0; i < c1; i++) {
                const SparseNode &nd = *children[i].src;
                tasks.push_back(ShrinkTask{nd.a, nd.b, nd.w, nd.w64, nd.m, nd.N, children[i].target, nd.k0, nd.idx,
                                           1 + children[i].h, lab.as<uint32_t>() + lo,
                                           kout.as<uint32_t>() + (i - c0)});
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
            // relabel, sort and merge every child's edges into a list of its own
            std::vector<MatBuf *> lists(B, nullptr);
            lo = 0;
            for (uint32_t b = 0; b < B && st == CAC_OK; b++) {
                const SparseNode &nd = *children[c0 + b].src;
                const uint64_t cap = std::max<uint64_t>(nd.m, 1);
                if ((st = eng.alloc(align_up(cap * 4) * 2 + align_up(cap * 8), &lists[b])) != CAC_OK) break;
                char *p = static_cast<char *>(lists[b]->p);
                uint32_t *oa = reinterpret_cast<uint32_t *>(p), *ob = reinterpret_cast<uint32_t *>(p + align_up(cap * 4));
                uint64_t *ow = reinterpret_cast<uint64_t *>(p + 2 * align_up(cap * 4));
                const uint32_t *lb = lab.as<uint32_t>() + lo;
                lo += nd.N;
                st = nd.w64 ? merge_edges<uint64_t>(ctx, nd.a, nd.b, static_cast<const uint64_t *>(nd.w), nd.m, lb,
                                                    kk[b], oa, ob, ow, counts.as<uint32_t>() + b, merge_scr.p)
                            : merge_edges<uint32_t>(ctx, nd.a, nd.b, static_cast<const uint32_t *>(nd.w), nd.m, lb,
                                                    kk[b], oa, ob, ow, counts.as<uint32_t>() + b, merge_scr.p);
            }
            if (st == CAC_OK && (cudaMemcpyAsync(mm.data(), counts.p, B * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                                 cudaStreamSynchronize(s) != cudaSuccess)) {
                set_error("sparse Karger-Stein: reading the merged edge counts failed");
                st = CAC_ERR_CUDA;
            }
            for (uint32_t b = 0; b < B; b++) {
                MatBuf *list = lists[b];
                if (!list) continue;
                list->refs++;  // held here until the child is placed
                if (st != CAC_OK) {
                    eng.release(list);
                    continue;
                }
                const SparseNode &nd = *children[c0 + b].src;
                const uint32_t k = kk[b];
                const uint64_t cap = std::max<uint64_t>(nd.m, 1);
                char *p = static_cast<char *>(list->p);
                const uint32_t *oa = reinterpret_cast<const uint32_t *>(p);
                const uint32_t *ob = reinterpret_cast<const uint32_t *>(p + align_up(cap * 4));
                const uint64_t *ow = reinterpret_cast<const uint64_t *>(p + 2 * align_up(cap * 4));
                if (mm[b] == 0 || k < 2) {
                    zero.assign(1, nd.cut);
                    st = zero_cuts(ctx, zero);
                } else if (ks_is_dense(ctx, k, mm[b])) {
                    MatBuf *mat = nullptr;
                    const uint64_t ld = ld_of(k), es = nd.small ? 4 : 8;
                    if ((st = eng.alloc(k * ld * es, &mat)) == CAC_OK) {
                        if (cudaMemsetAsync(mat->p, 0, k * ld * es, s) != cudaSuccess) {
                            set_error("sparse Karger-Stein: clearing a dense child failed");
                            st = CAC_ERR_CUDA;
                        } else if (nd.small) {
                            dense_from_pairs<uint32_t><<<grid_of(ctx, mm[b]), 256, 0, s>>>(
                                oa, ob, ow, mm[b], ld, static_cast<uint32_t *>(mat->p));
                        } else {
                            dense_from_pairs<uint64_t><<<grid_of(ctx, mm[b]), 256, 0, s>>>(
                                oa, ob, ow, mm[b], ld, static_cast<uint64_t *>(mat->p));
                        }
                        if (st == CAC_OK) {
                            eng.add(KNode{nd.cut, nd.k0, nd.idx, children[c0 + b].h, k, 0, nd.small, nd.query, mat->p,
                                          mat});
                        } else {
                            mat->refs++;  // a reference to drop: frees the matrix
                            eng.release(mat);
                        }
                    }
                } else {
                    list->refs++;  // the next level's node holds it
                    next.push_back(SparseNode{nd.cut, nd.k0, nd.idx, children[c0 + b].h, k, mm[b], oa, ob, ow, true,
                                              false, nd.small, nd.query, list});
                }
                eng.release(list);  // this scope's reference (the dense child's matrix is built)
            }
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
