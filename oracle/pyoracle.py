"""ORACLE (test infrastructure): ctypes binding of oracle/lib/liboracle.so.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import this module; it
checks the product and is never part of it. Build the library with ``make -C oracle``.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "lib", "liboracle.so")
        if not os.path.exists(path):
            raise RuntimeError("oracle library missing: run `make -C oracle` (or __graft_entry__.build())")
        L = ctypes.CDLL(path)
        L.orc_sitmo_block.argtypes = [_u64p, _u64p, _u64p]
        L.orc_sitmo_seed_output.argtypes = [ctypes.c_uint32, ctypes.c_uint64]
        L.orc_sitmo_seed_output.restype = ctypes.c_uint32
        L.orc_sitmo_outputs.argtypes = [_u64p, _u64p, ctypes.c_uint64, _u32p]
        L.orc_draw64.argtypes = [_u64p, ctypes.c_uint64, ctypes.c_uint64]
        L.orc_draw64.restype = ctypes.c_uint64
        L.orc_cc_labels.argtypes = [ctypes.c_uint32, ctypes.c_uint64, _u32p, _u32p, _u32p]
        L.orc_cc_labels.restype = ctypes.c_uint32
        L.orc_cc_iss.argtypes = [ctypes.c_uint32, ctypes.c_uint64, _u32p, _u32p, ctypes.c_uint32, ctypes.c_uint32,
                                 _u32p, _u32p]
        L.orc_cc_iss.restype = ctypes.c_uint32
        L.orc_cc_iss_mt.argtypes = [ctypes.c_uint32, ctypes.c_uint64, _u32p, _u32p, ctypes.c_uint32, ctypes.c_uint32,
                                    ctypes.c_uint32, _u32p, _u32p]
        L.orc_cc_iss_mt.restype = ctypes.c_uint32
        L.orc_cc_sample_count.argtypes = [ctypes.c_uint32, ctypes.c_uint64]
        L.orc_cc_sample_count.restype = ctypes.c_uint64
        L.orc_stoer_wagner_dense.argtypes = [ctypes.c_uint32, _u64p]
        L.orc_stoer_wagner_dense.restype = ctypes.c_uint64
        L.orc_exact_mincut.argtypes = [ctypes.c_uint32, ctypes.c_uint64, _u32p, _u32p, _u32p]
        L.orc_exact_mincut.restype = ctypes.c_uint64
        L.orc_ks_trial.argtypes = [ctypes.c_uint32, ctypes.c_uint64, _u32p, _u32p, _u32p, ctypes.c_uint32,
                                   ctypes.c_uint32]
        L.orc_ks_trial.restype = ctypes.c_uint64
        L.orc_set_dense_limit.argtypes = [ctypes.c_uint32]
        L.orc_set_dense_limit.restype = None
        L.orc_group_count.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
        L.orc_group_count.restype = ctypes.c_uint32
        L.orc_group_draws.argtypes = [ctypes.c_uint32]
        L.orc_group_draws.restype = ctypes.c_uint32
        L.orc_mincut_group_trial.argtypes = [ctypes.c_uint32, ctypes.c_uint64, _u32p, _u32p, _u32p, ctypes.c_uint32,
                                             ctypes.c_uint32]
        L.orc_mincut_group_trial.restype = ctypes.c_uint64
        L.orc_exact_mincut_noi.argtypes = [ctypes.c_uint32, ctypes.c_uint64, _u32p, _u32p, _u32p]
        L.orc_exact_mincut_noi.restype = ctypes.c_uint64
        L.orc_intermediate_size.argtypes = [ctypes.c_uint32, ctypes.c_uint64]
        L.orc_intermediate_size.restype = ctypes.c_uint32
        L.orc_number_of_trials.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_double]
        L.orc_number_of_trials.restype = ctypes.c_uint32
        L.orc_min_success_in_one_trial.argtypes = [ctypes.c_int]
        L.orc_min_success_in_one_trial.restype = ctypes.c_double
        L.orc_ks_target.argtypes = [ctypes.c_int]
        L.orc_ks_target.restype = ctypes.c_int
        L.orc_mincut_trial.argtypes = [ctypes.c_uint32, ctypes.c_uint64, _u32p, _u32p, _u32p, ctypes.c_uint32,
                                       ctypes.c_uint32, ctypes.c_uint32]
        L.orc_mincut_trial.restype = ctypes.c_uint64
        L.orc_ks_dense.argtypes = [ctypes.c_uint32, _u64p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32]
        L.orc_ks_dense.restype = ctypes.c_uint64
        L.orc_shrink_to_dense.argtypes = [ctypes.c_uint32, ctypes.c_uint64, _u32p, _u32p, _u32p, ctypes.c_uint32,
                                          ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _u64p]
        L.orc_shrink_to_dense.restype = ctypes.c_uint32
        L.orc_square_root.argtypes = [ctypes.c_uint32, ctypes.c_uint64, _u32p, _u32p, _u32p, ctypes.c_double,
                                      ctypes.c_uint32, ctypes.c_uint32, _u32p]
        L.orc_square_root.restype = ctypes.c_uint64
        L.orc_approx_trials.argtypes = [ctypes.c_double]
        L.orc_approx_trials.restype = ctypes.c_uint32
        L.orc_keep_threshold.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
        L.orc_keep_threshold.restype = ctypes.c_uint64
        L.orc_approx_cut.argtypes = [ctypes.c_uint32, ctypes.c_uint64, _u32p, _u32p, _u32p, ctypes.c_double,
                                     ctypes.c_uint32, ctypes.c_uint32, _u32p]
        L.orc_approx_cut.restype = ctypes.c_uint64
        L.orc_approx_cut_stream.argtypes = L.orc_approx_cut.argtypes
        L.orc_approx_cut_stream.restype = ctypes.c_uint64
        L.orc_ref_binomial_draws.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, _u32p, ctypes.c_uint32,
                                             ctypes.POINTER(ctypes.c_int32), _u32p]
        L.orc_ref_binomial_draws.restype = ctypes.c_int
        _LIB = L
    return _LIB


def _p32(a):
    return a.ctypes.data_as(_u32p)


def _p64(a):
    return a.ctypes.data_as(_u64p)


def _c32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def sitmo_block(key, ctr):
    k = np.array(key, dtype=np.uint64)
    c = np.array(ctr, dtype=np.uint64)
    out = np.zeros(4, dtype=np.uint64)
    lib().orc_sitmo_block(_p64(k), _p64(c), _p64(out))
    return out


def sitmo_outputs(key, ctr, count):
    k = np.array(key, dtype=np.uint64)
    c = np.array(ctr, dtype=np.uint64)
    out = np.zeros(count, dtype=np.uint32)
    lib().orc_sitmo_outputs(_p64(k), _p64(c), count, _p32(out))
    return out


def draw64(key, rnd, d):
    k = np.array(key, dtype=np.uint64)
    return int(lib().orc_draw64(_p64(k), rnd, d))


def cc_labels(n, u, v):
    u, v = _c32(u), _c32(v)
    labels = np.zeros(max(n, 1), dtype=np.uint32)
    count = lib().orc_cc_labels(n, len(u), _p32(u), _p32(v), _p32(labels))
    return int(count), labels[:n]


def cc_iss(n, u, v, seed, ranks=1, threads=1):
    """The reference's iterated-sparse-sampling CC loop over `ranks` ranks, their per-rank phases
    on `threads` host threads (same result for any thread count)."""
    u, v = _c32(u), _c32(v)
    labels = np.zeros(max(n, 1), dtype=np.uint32)
    rounds = np.zeros(1, dtype=np.uint32)
    count = lib().orc_cc_iss_mt(n, len(u), _p32(u), _p32(v), seed, ranks, threads, _p32(labels), _p32(rounds))
    return int(count), labels[:n], int(rounds[0])


def cc_sample_count(n, edges_left):
    return int(lib().orc_cc_sample_count(n, edges_left))


def stoer_wagner_dense(mat):
    m = np.ascontiguousarray(mat, dtype=np.uint64).copy()
    return int(lib().orc_stoer_wagner_dense(m.shape[0], _p64(m)))


def exact_mincut(n, u, v, w):
    u, v, w = _c32(u), _c32(v), _c32(w)
    return int(lib().orc_exact_mincut(n, len(u), _p32(u), _p32(v), _p32(w)))


def exact_mincut_noi(n, u, v, w):
    u, v, w = _c32(u), _c32(v), _c32(w)
    return int(lib().orc_exact_mincut_noi(n, len(u), _p32(u), _p32(v), _p32(w)))


def exact_mincut_many(graphs, threads=None):
    """Exact cuts of [(n, u, v, w), ...] on `threads` host threads (ctypes releases the GIL)."""
    import concurrent.futures as cf
    import os
    threads = threads or os.cpu_count() or 1
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        return list(ex.map(lambda g: exact_mincut_noi(*g), graphs))


def intermediate_size(n, m):
    return int(lib().orc_intermediate_size(n, m))


def number_of_trials(n, m, p):
    return int(lib().orc_number_of_trials(n, m, p))


def min_success_in_one_trial(n):
    return float(lib().orc_min_success_in_one_trial(n))


def ks_number_of_trials(n, p):
    """comincut::number_of_trials (src/karger-stein/co_mincut.cpp:44-73): the failure probability of
    one trial is multiplied in until it is at most 1 - p; one trial at n <= 128 or p == 0."""
    if n <= 128 or p == 0:
        return 1
    one = min_success_in_one_trial(n)
    failure, trials = 1.0, 0
    while failure > 1.0 - p:
        failure *= 1.0 - one
        trials += 1
    return trials


def set_dense_limit(n):
    """The vertex count above which Karger-Stein nodes stay edge lists (default 16384)."""
    lib().orc_set_dense_limit(n)


def ks_trial(n, u, v, w, seed, trial):
    u, v, w = _c32(u), _c32(v), _c32(w)
    return int(lib().orc_ks_trial(n, len(u), _p32(u), _p32(v), _p32(w), seed, trial))


def karger_stein(n, u, v, w, p, seed, threads=1):
    """Plain Karger-Stein on the whole graph (src/executables/karger_stein.cpp:34): trial i recurses
    from the root with the counter-addressed draws of (seed, rank 0, trial i) -- the dense n x n
    matrix, or the edge list when the graph is sparse (n above the dense limit, or fewer than
    n^2 / 32 edges above 2048 vertices); the answer is the minimum over ks_number_of_trials(n, p)
    trials. Returns (cut, trials)."""
    trials = ks_number_of_trials(n, p)
    if n < 2:
        return 0, trials
    if threads > 1:
        import concurrent.futures as cf
        with cf.ThreadPoolExecutor(max_workers=threads) as ex:
            vals = list(ex.map(lambda i: ks_trial(n, u, v, w, seed, i), range(trials)))
    else:
        vals = [ks_trial(n, u, v, w, seed, i) for i in range(trials)]
    return min(vals), trials


def group_count(ranks, trials):
    """Trials of SquareRootCut's high-concurrency variant: ranks / 2^floor(log2(ranks / trials))."""
    return int(lib().orc_group_count(ranks, trials))


def group_draws(n):
    return int(lib().orc_group_draws(n))


def mincut_group_trial(n, u, v, w, seed, group):
    """One trial of the high-concurrency group variant (see oracle/mincut.c)."""
    u, v, w = _c32(u), _c32(v), _c32(w)
    return int(lib().orc_mincut_group_trial(n, len(u), _p32(u), _p32(v), _p32(w), seed, group))


def ks_target(n):
    return int(lib().orc_ks_target(n))


def mincut_trial(n, u, v, w, seed, rank, trial):
    u, v, w = _c32(u), _c32(v), _c32(w)
    return int(lib().orc_mincut_trial(n, len(u), _p32(u), _p32(v), _p32(w), seed, rank, trial))


def ks_dense(mat, seed, rank, trial):
    m = np.ascontiguousarray(mat, dtype=np.uint64)
    return int(lib().orc_ks_dense(m.shape[0], _p64(m), seed, rank, trial))


def shrink_to_dense(n, u, v, w, target, seed, rank, trial):
    u, v, w = _c32(u), _c32(v), _c32(w)
    out = np.zeros(max(n, 1) * max(n, 1), dtype=np.uint64)
    k = lib().orc_shrink_to_dense(n, len(u), _p32(u), _p32(v), _p32(w), target, seed, rank, trial, _p64(out))
    return int(k), out[: k * k].reshape(k, k)


def square_root(n, u, v, w, p, seed, ranks=1):
    u, v, w = _c32(u), _c32(v), _c32(w)
    per = np.zeros(1, dtype=np.uint32)
    cut = lib().orc_square_root(n, len(u), _p32(u), _p32(v), _p32(w), p, seed, ranks, _p32(per))
    return int(cut), int(per[0])


def approx_trials(p):
    return int(lib().orc_approx_trials(p))


def keep_threshold(level, w):
    return int(lib().orc_keep_threshold(level, w))


def approx_cut(n, u, v, w, p, seed, ranks=1):
    u, v, w = _c32(u), _c32(v), _c32(w)
    lv = np.zeros(1, dtype=np.uint32)
    cut = lib().orc_approx_cut(n, len(u), _p32(u), _p32(v), _p32(w), p, seed, ranks, _p32(lv))
    return int(cut), int(lv[0])


def approx_cut_stream(n, u, v, w, p, seed, ranks=1):
    """approx_cut on the reference's own draws (sitmo::prng_engine(seed + r) through libstdc++'s
    binomial_distribution, src/ApproximateCut.cpp:33-58). Returns (cut, level); None where a draw
    leaves the restated regime (weight * 2^-level >= 8)."""
    u, v, w = _c32(u), _c32(v), _c32(w)
    lv = np.zeros(1, dtype=np.uint32)
    cut = lib().orc_approx_cut_stream(n, len(u), _p32(u), _p32(v), _p32(w), p, seed, ranks, _p32(lv))
    return None if cut == 0 else (int(cut), int(lv[0]))


def ref_binomial_draws(seed, level, count, weights):
    """`count` draws binomial_distribution<int>(weights[k % len], 2^-level) on
    sitmo::prng_engine(seed), and the engine's next raw output."""
    w = _c32(weights)
    out = np.zeros(max(count, 1), dtype=np.int32)
    nxt = np.zeros(1, dtype=np.uint32)
    st = lib().orc_ref_binomial_draws(seed, level, count, _p32(w), len(w),
                                      out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _p32(nxt))
    return None if st else (out[:count].tolist(), int(nxt[0]))
