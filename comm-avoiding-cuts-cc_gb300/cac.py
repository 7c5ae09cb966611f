"""Python host mirror of libcac's C ABI (include/cac.h), loaded with ctypes.

Mirrors the reference's callable classes for this path:
  * ``connected_components``  UnweightedIteratedSparseSampling::connectedComponents
                              (src/UnweightedIteratedSparseSampling.cpp:40-72)
  * ``square_root``           SquareRootCut::runMaster (src/SquareRootCut.cpp:15-25)
  * ``approx_cut``            ApproximateCut::run (src/ApproximateCut.cpp:10-79)
Every non-zero status of the library raises ``CacError`` (the reference throws or asserts).
There is no fallback: if libcac.so is missing or no CUDA device is present, calls fail loudly.
"""
import ctypes
import os
import weakref
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libcac.so")

HOST, DEVICE = 0, 1
_STATUS = {0: "ok", -1: "invalid argument", -2: "out of device memory or HBM budget", -3: "malformed input",
           -4: "CUDA runtime error", -5: "device-side bound exceeded", -6: "unsupported", -7: "I/O error"}


class CacError(RuntimeError):
    def __init__(self, status, where, detail):
        super().__init__("%s failed: %s (%d): %s" % (where, _STATUS.get(status, "?"), status, detail))
        self.status = status


class _Config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("stream", ctypes.c_void_p), ("hbm_budget_bytes", ctypes.c_uint64)]


class CCResult(ctypes.Structure):
    _fields_ = [("num_components", ctypes.c_uint32), ("rounds", ctypes.c_uint32), ("sampled_edges", ctypes.c_uint64),
                ("device_ms", ctypes.c_float), ("edge_pass_ms", ctypes.c_float), ("sample_ms", ctypes.c_float),
                ("hook_ms", ctypes.c_float), ("label_ms", ctypes.c_float)]


class MincutResult(ctypes.Structure):
    _fields_ = [("cut", ctypes.c_uint64), ("trials_per_rank", ctypes.c_uint32), ("total_trials", ctypes.c_uint32),
                ("intermediate", ctypes.c_uint32), ("high_concurrency", ctypes.c_uint32),
                ("device_ms", ctypes.c_float)]


class MincutQuery(ctypes.Structure):
    _fields_ = [("graph", ctypes.c_void_p), ("success_probability", ctypes.c_double), ("seed", ctypes.c_uint32),
                ("virtual_ranks", ctypes.c_uint32)]


class ApproxResult(ctypes.Structure):
    _fields_ = [("cut", ctypes.c_uint64), ("trials", ctypes.c_uint32), ("copies", ctypes.c_uint32),
                ("level", ctypes.c_uint32), ("device_ms", ctypes.c_float)]


class GenSpec(ctypes.Structure):
    _fields_ = [("family", ctypes.c_int), ("n", ctypes.c_uint32), ("p", ctypes.c_double),
                ("avg_degree", ctypes.c_double), ("k", ctypes.c_uint32), ("scale", ctypes.c_uint32),
                ("edge_factor", ctypes.c_uint32), ("a", ctypes.c_double), ("b", ctypes.c_double),
                ("c", ctypes.c_double), ("seed", ctypes.c_uint32), ("wmin", ctypes.c_uint32), ("wmax", ctypes.c_uint32)]


GEN_FAMILIES = {"erdos_renyi": 1, "erdos_renyi_m": 2, "watts_strogatz": 3, "rmat": 4, "complete": 5}


class _ServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_uint64)]


class Request(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("graph", ctypes.c_void_p), ("success_probability", ctypes.c_double),
                ("seed", ctypes.c_uint32), ("virtual_ranks", ctypes.c_uint32), ("labels_host", ctypes.c_void_p)]


class Response(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("cut", ctypes.c_uint64), ("trials", ctypes.c_uint32),
                ("num_components", ctypes.c_uint32), ("queue_ms", ctypes.c_double), ("service_ms", ctypes.c_double),
                ("message", ctypes.c_char * 160)]


QUERY_MINCUT, QUERY_APPROX, QUERY_CC = 1, 2, 3
PENDING = 1

_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_vp = ctypes.c_void_p
_LIB = None

# (name, restype, argtypes) of every exported entry point declared in include/cac.h
EXPORTS = [
    ("cac_ctx_create", ctypes.c_int, [ctypes.POINTER(_Config), ctypes.POINTER(_vp)]),
    ("cac_ctx_destroy", ctypes.c_int, [_vp]),
    ("cac_ctx_set_dense_limit", ctypes.c_int, [_vp, ctypes.c_uint32]),
    ("cac_ctx_set_quotient_kernel", ctypes.c_int, [_vp, ctypes.c_int]),
    ("cac_ctx_set_plan_ahead", ctypes.c_int, [_vp, ctypes.c_int]),
    ("cac_ctx_plan_redos", ctypes.c_uint64, [_vp]),
    ("cac_error_string", ctypes.c_char_p, [ctypes.c_int]),
    ("cac_last_error", ctypes.c_char_p, []),
    ("cac_ctx_device_bytes", ctypes.c_uint64, [_vp]),
    ("cac_graph_load_file", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.POINTER(_vp)]),
    ("cac_graph_from_edges", ctypes.c_int, [_vp, ctypes.c_uint32, ctypes.c_uint64, _vp, _vp, _vp, ctypes.c_int,
                                            ctypes.POINTER(_vp)]),
    ("cac_graph_free", ctypes.c_int, [_vp]),
    ("cac_graph_info", ctypes.c_int, [_vp, _u32p, _u64p, _u64p]),
    ("cac_graph_copy_edges", ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int]),
    ("cac_parse_file", ctypes.c_int, [ctypes.c_char_p, _u32p, _u64p, _vp, _vp, _vp, ctypes.c_uint64]),
    ("cac_parse_header", ctypes.c_int, [ctypes.c_char_p, _u32p, _u64p]),
    ("cac_cache_write", ctypes.c_int, [ctypes.c_char_p, ctypes.c_uint32, ctypes.c_uint64, _vp, _vp, _vp]),
    ("cac_cache_convert", ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p]),
    ("cac_cc", ctypes.c_int, [_vp, _vp, ctypes.c_uint32, ctypes.c_uint32, _vp, ctypes.c_int,
                              ctypes.POINTER(CCResult)]),
    ("cac_cc_edges", ctypes.c_int, [_vp, ctypes.c_uint32, ctypes.c_uint64, _vp, _vp, ctypes.c_uint32,
                                    ctypes.c_uint32, _vp, ctypes.POINTER(CCResult)]),
    ("cac_cc_noalloc", ctypes.c_int, [ctypes.c_uint32, ctypes.c_uint64, _vp, _vp, _vp, _vp, _vp]),
    ("cac_mincut", ctypes.c_int, [_vp, _vp, ctypes.c_double, ctypes.c_uint32, ctypes.c_uint32,
                                  ctypes.POINTER(MincutResult)]),
    ("cac_mincut_batch", ctypes.c_int, [_vp, _vp, ctypes.c_uint32, _vp]),
    ("cac_karger_stein", ctypes.c_int, [_vp, _vp, ctypes.c_double, ctypes.c_uint32, ctypes.POINTER(MincutResult)]),
    ("cac_mincut_trials", ctypes.c_int, [_vp, _vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _vp]),
    ("cac_karger_stein_trials", ctypes.c_int, [_vp, _vp, ctypes.c_uint32, ctypes.c_uint32, _vp]),
    ("cac_mincut_group_trials", ctypes.c_int, [_vp, _vp, ctypes.c_uint32, ctypes.c_uint32, _vp]),
    ("cac_ks_dense", ctypes.c_int, [_vp, ctypes.c_uint32, _vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                    _u64p]),
    ("cac_exact_cut_small", ctypes.c_int, [_vp, ctypes.c_uint32, _vp, _u64p]),
    ("cac_approx_cut", ctypes.c_int, [_vp, _vp, ctypes.c_double, ctypes.c_uint32, ctypes.c_uint32,
                                      ctypes.POINTER(ApproxResult)]),
    ("cac_approx_cut_seed_replay", ctypes.c_int, [_vp, _vp, ctypes.c_double, ctypes.c_uint32, ctypes.c_uint32,
                                      ctypes.POINTER(ApproxResult)]),
    ("cac_sitmo_blocks", ctypes.c_int, [_vp, _u64p, _u64p, ctypes.c_uint64, _vp]),
    ("cac_graph_generate", ctypes.c_int, [_vp, ctypes.POINTER(GenSpec), ctypes.POINTER(_vp)]),
    ("cac_click_edges", ctypes.c_int, [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _vp, _vp, _vp,
                                       ctypes.c_uint64, _u64p]),
    ("cac_graph_click", ctypes.c_int, [_vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(_vp)]),
    ("cac_server_create", ctypes.c_int, [ctypes.POINTER(_ServerConfig), ctypes.POINTER(_vp)]),
    ("cac_server_graph", ctypes.c_int, [_vp, ctypes.c_uint32, ctypes.c_uint64, _vp, _vp, _vp, ctypes.POINTER(_vp)]),
    ("cac_server_generate", ctypes.c_int, [_vp, ctypes.POINTER(GenSpec), ctypes.POINTER(_vp)]),
    ("cac_server_submit", ctypes.c_int, [_vp, ctypes.POINTER(Request), _u64p]),
    ("cac_server_poll", ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(Response)]),
    ("cac_server_destroy", ctypes.c_int, [_vp]),
]


def lib():
    """Load libcac.so (raises if it was not built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libcac.so not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in EXPORTS:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def _check(status, where):
    if status != 0:
        raise CacError(status, where, lib().cac_last_error().decode(errors="replace"))


def _ptr(a):
    """Host numpy array or device tensor-like (with data_ptr) -> (pointer, where)."""
    if a is None:
        return None, HOST
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr()), (DEVICE if getattr(a, "is_cuda", False) else HOST)
    return ctypes.c_void_p(a.ctypes.data), HOST


class Context:
    """One device + one CUDA stream (cac_ctx). `stream` is a raw cudaStream_t handle (int) or None."""

    def __init__(self, device=0, stream=None, hbm_budget_bytes=0):
        cfg = _Config(device, ctypes.c_void_p(stream) if stream else None, hbm_budget_bytes)
        h = _vp()
        _check(lib().cac_ctx_create(ctypes.byref(cfg), ctypes.byref(h)), "cac_ctx_create")
        self.h = h
        self._graphs = weakref.WeakSet()

    def set_dense_limit(self, max_dense_vertices):
        """Karger-Stein nodes above this many vertices (or sparse ones above 2048) stay edge lists."""
        _check(lib().cac_ctx_set_dense_limit(self.h, max_dense_vertices), "cac_ctx_set_dense_limit")

    def set_plan_ahead(self, enabled):
        """Karger-Stein levels planned at their target sizes (default) or read back level by level."""
        _check(lib().cac_ctx_set_plan_ahead(self.h, 1 if enabled else 0), "cac_ctx_set_plan_ahead")

    def plan_redos(self):
        """Runs redone level by level after a child stopped off its planned size."""
        return int(lib().cac_ctx_plan_redos(self.h))

    def set_quotient_kernel(self, kind):
        """0: autotuned; 1 warp per row; 2 eight warps per row; 3 warp per row with bulk-copy staging;
        4 the fixed size rule (eight warps per row from N = 2000 on), without timing."""
        _check(lib().cac_ctx_set_quotient_kernel(self.h, kind), "cac_ctx_set_quotient_kernel")

    def close(self):
        if self.h:
            for g in list(self._graphs):
                g.free()
            lib().cac_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def device_bytes(self):
        return int(lib().cac_ctx_device_bytes(self.h))

    # ---- graphs ----
    def graph(self, n, u, v, w=None):
        """Upload an edge list (numpy uint32 host arrays or CUDA tensors) as a device graph."""
        if not hasattr(u, "data_ptr"):
            u = np.ascontiguousarray(u, dtype=np.uint32)
            v = np.ascontiguousarray(v, dtype=np.uint32)
            w = None if w is None else np.ascontiguousarray(w, dtype=np.uint32)
        pu, where = _ptr(u)
        pv, _ = _ptr(v)
        pw, _ = _ptr(w)
        h = _vp()
        _check(lib().cac_graph_from_edges(self.h, n, len(u), pu, pv, pw, where, ctypes.byref(h)),
               "cac_graph_from_edges")
        g = Graph(self, h, (u, v, w))
        self._graphs.add(g)
        return g

    def generate(self, family, seed=0, n=0, p=0.0, avg_degree=0.0, k=0, scale=0, edge_factor=0,
                 a=0.57, b=0.19, c=0.19, wmin=1, wmax=1):
        """A seeded synthetic graph made on the device; the same edges as graphgen.<family>."""
        spec = GenSpec(GEN_FAMILIES[family], n, p, avg_degree, k, scale, edge_factor, a, b, c, seed, wmin, wmax)
        h = _vp()
        _check(lib().cac_graph_generate(self.h, ctypes.byref(spec), ctypes.byref(h)), "cac_graph_generate")
        g = Graph(self, h, None)
        self._graphs.add(g)
        return g

    def click(self, n, virtual_ranks=1, seed=0):
        """The reference's CLICK graph on the device (cac_graph_click)."""
        h = _vp()
        _check(lib().cac_graph_click(self.h, n, virtual_ranks, seed, ctypes.byref(h)), "cac_graph_click")
        g = Graph(self, h, None)
        self._graphs.add(g)
        return g

    def load(self, path):
        h = _vp()
        _check(lib().cac_graph_load_file(self.h, path.encode(), ctypes.byref(h)), "cac_graph_load_file")
        g = Graph(self, h, None)
        self._graphs.add(g)
        return g

    # ---- primitives ----
    def sitmo_blocks(self, key, ctr0, nblocks):
        k = np.array(key, dtype=np.uint64)
        c = np.array(ctr0, dtype=np.uint64)
        out = np.zeros(4 * nblocks, dtype=np.uint64)
        _check(lib().cac_sitmo_blocks(self.h, k.ctypes.data_as(_u64p), c.ctypes.data_as(_u64p), nblocks,
                                      ctypes.c_void_p(out.ctypes.data)), "cac_sitmo_blocks")
        return out.reshape(nblocks, 4)

    def cc_edges(self, n, u, v, seed=0, virtual_ranks=1, labels=None):
        """One-call CC from host edge arrays to host labels (copies included)."""
        res = CCResult()
        pl = None if labels is None else ctypes.c_void_p(labels.ctypes.data)
        _check(lib().cac_cc_edges(self.h, n, len(u), ctypes.c_void_p(u.ctypes.data), ctypes.c_void_p(v.ctypes.data),
                                  seed, virtual_ranks, pl, ctypes.byref(res)), "cac_cc_edges")
        return res

    def ks_dense(self, mat, seed, rank, trial):
        m = np.ascontiguousarray(mat, dtype=np.uint64)
        out = ctypes.c_uint64()
        _check(lib().cac_ks_dense(self.h, m.shape[0], ctypes.c_void_p(m.ctypes.data), seed, rank, trial,
                                  ctypes.byref(out)), "cac_ks_dense")
        return int(out.value)

    def mincut_batch(self, graphs, success_probability=0.95, seeds=None, virtual_ranks=1):
        """square_root on many graphs in one batch -> list of MincutResult (same values as one by one)."""
        k = len(graphs)
        qs = (MincutQuery * max(k, 1))()
        for i, g in enumerate(graphs):
            qs[i] = MincutQuery(g.h, success_probability, 0 if seeds is None else seeds[i], virtual_ranks)
        res = (MincutResult * max(k, 1))()
        _check(lib().cac_mincut_batch(self.h, ctypes.cast(qs, ctypes.c_void_p), k, ctypes.cast(res, ctypes.c_void_p)),
               "cac_mincut_batch")
        return [res[i] for i in range(k)]

    def exact_cut_small(self, mat):
        m = np.ascontiguousarray(mat, dtype=np.uint64)
        out = ctypes.c_uint64()
        _check(lib().cac_exact_cut_small(self.h, m.shape[0], ctypes.c_void_p(m.ctypes.data), ctypes.byref(out)),
               "cac_exact_cut_small")
        return int(out.value)


class Graph:
    def __init__(self, ctx, h, keepalive, queries=True):
        self.ctx = ctx if queries else None
        self._owner = ctx
        self.h = h
        self._keep = keepalive
        n, m, w = ctypes.c_uint32(), ctypes.c_uint64(), ctypes.c_uint64()
        _check(lib().cac_graph_info(h, ctypes.byref(n), ctypes.byref(m), ctypes.byref(w)), "cac_graph_info")
        self.n, self.m, self.total_weight = int(n.value), int(m.value), int(w.value)

    def free(self):
        if self.h and self._owner.h:
            lib().cac_graph_free(self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def edges(self):
        """-> (u, v, w) host copies of the device edge arrays."""
        k = max(self.m, 1)
        u, v, w = np.zeros(k, np.uint32), np.zeros(k, np.uint32), np.zeros(k, np.uint32)
        _check(lib().cac_graph_copy_edges(self.h, ctypes.c_void_p(u.ctypes.data), ctypes.c_void_p(v.ctypes.data),
                                          ctypes.c_void_p(w.ctypes.data), HOST), "cac_graph_copy_edges")
        return u[: self.m], v[: self.m], w[: self.m]

    # UnweightedIteratedSparseSampling::connectedComponents
    def connected_components(self, seed=0, virtual_ranks=1, labels=True, out=None):
        """Returns (number_of_components, labels or None, CCResult). `out` may be a device
        tensor (or host array) of n uint32 that receives the labels."""
        res = CCResult()
        if out is not None:
            pl, where = _ptr(out)
        elif labels:
            out = np.zeros(max(self.n, 1), dtype=np.uint32)
            pl, where = _ptr(out)
        else:
            pl, where = None, HOST
        _check(lib().cac_cc(self.ctx.h, self.h, seed, virtual_ranks, pl, where, ctypes.byref(res)), "cac_cc")
        lab = None
        if out is not None and not hasattr(out, "data_ptr"):
            lab = out[: self.n]
        elif out is not None:
            lab = out
        return int(res.num_components), lab, res

    # SquareRootCut::runMaster
    def square_root(self, success_probability=0.95, seed=0, virtual_ranks=1):
        res = MincutResult()
        _check(lib().cac_mincut(self.ctx.h, self.h, success_probability, seed, virtual_ranks, ctypes.byref(res)),
               "cac_mincut")
        return res

    # comincut::minimum_cut (the karger_stein executable)
    def karger_stein(self, success_probability=0.9, seed=0):
        res = MincutResult()
        _check(lib().cac_karger_stein(self.ctx.h, self.h, success_probability, seed, ctypes.byref(res)),
               "cac_karger_stein")
        return res

    def karger_stein_trials(self, seed, trials):
        """Every trial's value of plain Karger-Stein (trials 0 .. trials - 1)."""
        out = np.zeros(max(trials, 1), dtype=np.uint64)
        _check(lib().cac_karger_stein_trials(self.ctx.h, self.h, seed, trials, ctypes.c_void_p(out.ctypes.data)),
               "cac_karger_stein_trials")
        return out[:trials]

    def group_trials(self, seed, groups):
        """Every group's value of square_root's group variant (groups 0 .. groups - 1)."""
        out = np.zeros(max(groups, 1), dtype=np.uint64)
        _check(lib().cac_mincut_group_trials(self.ctx.h, self.h, seed, groups, ctypes.c_void_p(out.ctypes.data)),
               "cac_mincut_group_trials")
        return out[:groups]

    def trials(self, seed, virtual_ranks, trials_per_rank):
        out = np.zeros(virtual_ranks * trials_per_rank, dtype=np.uint64)
        _check(lib().cac_mincut_trials(self.ctx.h, self.h, seed, virtual_ranks, trials_per_rank,
                                       ctypes.c_void_p(out.ctypes.data)), "cac_mincut_trials")
        return out.reshape(virtual_ranks, trials_per_rank)

    # ApproximateCut::run
    def approx_cut(self, success_probability=0.9, seed=0, virtual_ranks=1, seed_replay=False):
        """seed_replay: draw the reference's own random numbers (sitmo(seed + r) through
        libstdc++'s binomial_distribution), so the answer equals the reference executable's;
        unit edge weights only."""
        res = ApproxResult()
        fn, name = ((lib().cac_approx_cut_seed_replay, "cac_approx_cut_seed_replay") if seed_replay
                    else (lib().cac_approx_cut, "cac_approx_cut"))
        _check(fn(self.ctx.h, self.h, success_probability, seed, virtual_ranks, ctypes.byref(res)), name)
        return res


class Server:
    """Serving loop (cac_server): graphs stay resident; square_root, approx_cut and parallel_cc
    queries are submitted as they arrive and answered with the values of the single-query calls."""

    def __init__(self, device=0, hbm_budget_bytes=0):
        h = _vp()
        _check(lib().cac_server_create(ctypes.byref(_ServerConfig(device, hbm_budget_bytes)), ctypes.byref(h)),
               "cac_server_create")
        self.h = h
        self._graphs = weakref.WeakSet()
        self._labels = {}

    def graph(self, n, u, v, w=None):
        u = np.ascontiguousarray(u, dtype=np.uint32)
        v = np.ascontiguousarray(v, dtype=np.uint32)
        w = None if w is None else np.ascontiguousarray(w, dtype=np.uint32)
        h = _vp()
        _check(lib().cac_server_graph(self.h, n, len(u), ctypes.c_void_p(u.ctypes.data), ctypes.c_void_p(v.ctypes.data),
                                      None if w is None else ctypes.c_void_p(w.ctypes.data), ctypes.byref(h)),
               "cac_server_graph")
        g = Graph(self, h, None, queries=False)
        self._graphs.add(g)
        return g

    def generate(self, family, seed=0, n=0, p=0.0, avg_degree=0.0, k=0, scale=0, edge_factor=0,
                 a=0.57, b=0.19, c=0.19, wmin=1, wmax=1):
        spec = GenSpec(GEN_FAMILIES[family], n, p, avg_degree, k, scale, edge_factor, a, b, c, seed, wmin, wmax)
        h = _vp()
        _check(lib().cac_server_generate(self.h, ctypes.byref(spec), ctypes.byref(h)), "cac_server_generate")
        g = Graph(self, h, None, queries=False)
        self._graphs.add(g)
        return g

    def submit(self, kind, graph, success_probability=0.0, seed=0, virtual_ranks=1, labels=False):
        """-> ticket. kind: "square_root", "approx_cut" or "parallel_cc"."""
        k = {"square_root": QUERY_MINCUT, "approx_cut": QUERY_APPROX, "parallel_cc": QUERY_CC}[kind]
        out = np.zeros(max(graph.n, 1), np.uint32) if (labels and k == QUERY_CC) else None
        req = Request(k, graph.h, success_probability, seed, virtual_ranks,
                      None if out is None else ctypes.c_void_p(out.ctypes.data))
        t = ctypes.c_uint64()
        _check(lib().cac_server_submit(self.h, ctypes.byref(req), ctypes.byref(t)), "cac_server_submit")
        if out is not None:
            self._labels[int(t.value)] = out[: graph.n]
        return int(t.value)

    def poll(self, ticket, wait=True):
        """-> (Response, labels or None), or None while pending (wait=False). A failed query raises."""
        r = Response()
        st = lib().cac_server_poll(self.h, ticket, 1 if wait else 0, ctypes.byref(r))
        if st == PENDING:
            return None
        _check(st, "cac_server_poll")
        labels = self._labels.pop(ticket, None)
        if r.status != 0:
            raise CacError(r.status, "server query %d" % ticket, r.message.decode(errors="replace"))
        return r, labels

    def close(self):
        if self.h:
            lib().cac_server_destroy(self.h)  # frees the server's graphs too
            for g in list(self._graphs):
                g.h = None
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def click_edges(n, virtual_ranks=1, seed=0):
    """The reference's CLICK graph (host code, no device) -> (n, u, v, w)."""
    m = ctypes.c_uint64()
    _check(lib().cac_click_edges(n, virtual_ranks, seed, None, None, None, 0, ctypes.byref(m)), "cac_click_edges")
    k = int(m.value)
    u, v, w = (np.zeros(max(k, 1), np.uint32) for _ in range(3))
    _check(lib().cac_click_edges(n, virtual_ranks, seed, ctypes.c_void_p(u.ctypes.data), ctypes.c_void_p(v.ctypes.data),
                                 ctypes.c_void_p(w.ctypes.data), k, ctypes.byref(m)), "cac_click_edges")
    return n, u[:k], v[:k], w[:k]


def parse_file(path):
    """Parse an edge-list file with the library's reader -> (n, u, v, w)."""
    n, m = ctypes.c_uint32(), ctypes.c_uint64()
    _check(lib().cac_parse_header(path.encode(), ctypes.byref(n), ctypes.byref(m)), "cac_parse_header")
    cap = int(m.value)
    u = np.zeros(max(cap, 1), np.uint32)
    v = np.zeros(max(cap, 1), np.uint32)
    w = np.zeros(max(cap, 1), np.uint32)
    _check(lib().cac_parse_file(path.encode(), ctypes.byref(n), ctypes.byref(m), ctypes.c_void_p(u.ctypes.data),
                                ctypes.c_void_p(v.ctypes.data), ctypes.c_void_p(w.ctypes.data), cap),
           "cac_parse_file")
    k = int(m.value)
    return int(n.value), u[:k], v[:k], w[:k]


def cache_write(path, n, u, v, w=None):
    """Binary cache of an edge list (host arrays; w None: unweighted, read back as weights 1)."""
    u = np.ascontiguousarray(u, dtype=np.uint32)
    v = np.ascontiguousarray(v, dtype=np.uint32)
    pw = None
    if w is not None:
        w = np.ascontiguousarray(w, dtype=np.uint32)
        pw = ctypes.c_void_p(w.ctypes.data)
    _check(lib().cac_cache_write(path.encode(), n, len(u), ctypes.c_void_p(u.ctypes.data),
                                 ctypes.c_void_p(v.ctypes.data), pw), "cac_cache_write")


def cache_convert(input_path, cache_path):
    """Parses a text edge list and writes its binary cache."""
    _check(lib().cac_cache_convert(input_path.encode(), cache_path.encode()), "cac_cache_convert")
