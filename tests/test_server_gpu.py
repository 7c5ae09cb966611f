"""Serving loop (cac_server): square_root, approx_cut and parallel_cc queries submitted from several
threads while others run; every response equals the single-query entry point's answer and the
oracle's, whatever else was in flight. Errors of one query are reported in its response only."""
import threading

import numpy as np
import pytest

import graphgen
import pyoracle as O

pytestmark = pytest.mark.gpu


def _graphs():
    specs = [graphgen.erdos_renyi_m(90, 10.0, 1, wmax=50),
             graphgen.watts_strogatz(300, 10, 0.3, 2, wmax=100),
             graphgen.erdos_renyi(200, 0.08, 3),
             graphgen.erdos_renyi_m(1500, 12.0, 4, wmax=100),  # Stage 1 pre-contraction (t < n)
             graphgen.barabasi_albert(5000, 4, 5)]
    return specs


def _queries(count, graphs, seed=7):
    rng = np.random.default_rng(seed)
    kinds = ["square_root", "approx_cut", "parallel_cc"]
    out = []
    for i in range(count):
        gi = int(rng.integers(len(graphs)))
        kind = kinds[i % 3] if gi < 4 else "parallel_cc"
        p = 0.9 if kind != "approx_cut" else 0.8
        out.append((kind, gi, p, int(rng.integers(1000)), int(rng.integers(1, 4))))
    return out


def _single(ctx_graph, kind, p, seed, ranks):
    if kind == "square_root":
        r = ctx_graph.square_root(p, seed=seed, virtual_ranks=ranks)
        return int(r.cut), int(r.trials_per_rank)
    if kind == "approx_cut":
        r = ctx_graph.approx_cut(p, seed=seed, virtual_ranks=ranks)
        return int(r.cut), int(r.trials)
    c, lab, _ = ctx_graph.connected_components(seed=seed, virtual_ranks=ranks)
    return c, lab.copy()


def test_mixed_stream_matches_single_queries(libcac, ctx):
    specs = _graphs()
    qs = _queries(36, specs)
    singles = [ctx.graph(*s) for s in specs]
    expect = [_single(singles[gi], kind, p, sd, rk) for kind, gi, p, sd, rk in qs]
    with libcac.Server(0) as srv:
        sg = [srv.graph(*s) for s in specs]
        tickets = [None] * len(qs)

        def submit(part):
            for i in range(part, len(qs), 2):
                kind, gi, p, sd, rk = qs[i]
                tickets[i] = srv.submit(kind, sg[gi], p, sd, rk, labels=(kind == "parallel_cc"))

        th = [threading.Thread(target=submit, args=(k,)) for k in range(2)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        for i, (kind, gi, p, sd, rk) in enumerate(qs):
            resp, labels = srv.poll(tickets[i])
            assert resp.queue_ms >= 0 and resp.service_ms >= 0
            if kind == "parallel_cc":
                assert resp.num_components == expect[i][0]
                assert np.array_equal(labels, expect[i][1])
            else:
                assert (int(resp.cut), int(resp.trials)) == expect[i], (kind, gi, sd, rk)
    # the square_root answers are the exact minimum cuts, the CC labels the reference's
    for i, (kind, gi, p, sd, rk) in enumerate(qs):
        n, u, v, w = specs[gi]
        if kind == "square_root":
            assert expect[i][0] == O.exact_mincut(n, u, v, w)
        elif kind == "parallel_cc":
            count, labels = O.cc_labels(n, u, v)
            assert expect[i][0] == count and np.array_equal(expect[i][1], labels)


def _estimate(n, m, p):
    """The server's admission estimate of one square_root query (roots and two more levels)."""
    t = O.intermediate_size(n, m)
    trials = O.number_of_trials(n, m, p)
    tt = min(t, n)
    return (trials if t < n else 1) * tt * tt * 8 * 3 + trials * 8


def test_small_budget_serialises_but_keeps_values(libcac, ctx):
    specs = _graphs()[:3]
    singles = [ctx.graph(*s) for s in specs]
    est = [_estimate(n, len(u), 0.95) for n, u, _, _ in specs]
    budget = max(est) + (1 << 20)  # each query fits alone, not all together
    assert sum(est) > budget
    with libcac.Server(0, hbm_budget_bytes=budget) as srv:
        sg = [srv.graph(*s) for s in specs]
        tickets = [srv.submit("square_root", g, 0.95, seed=i) for i, g in enumerate(sg)]
        for i, t in enumerate(tickets):
            resp, _ = srv.poll(t)
            alone = singles[i].square_root(0.95, seed=i)
            assert resp.cut == alone.cut and resp.trials == alone.trials_per_rank


def test_poll_without_wait_and_unknown_ticket(libcac):
    n, u, v, w = graphgen.erdos_renyi(120, 0.1, 9)
    with libcac.Server(0) as srv:
        g = srv.graph(n, u, v, w)
        t = srv.submit("square_root", g, 0.9, seed=1)
        got = None
        while got is None:
            got = srv.poll(t, wait=False)
        assert got[0].cut == O.exact_mincut(n, u, v, w)
        with pytest.raises(libcac.CacError):
            srv.poll(t)  # retired
        with pytest.raises(libcac.CacError):
            srv.submit("square_root", g, 1.5)


def test_large_sparse_graph_in_the_mix(libcac, ctx):
    # 20000 vertices with sparse pre-contraction (global-memory Stage 1) served between small queries
    n, u, v, w = graphgen.watts_strogatz(20000, 4, 0.3, 8, wmax=100)
    ns, us, vs, ws = graphgen.erdos_renyi(150, 0.1, 4)
    want = ctx.graph(n, u, v, w).square_root(0.5, seed=2)
    with libcac.Server(0) as srv:
        gb, gs = srv.graph(n, u, v, w), srv.graph(ns, us, vs, ws)
        t0 = srv.submit("square_root", gs, 0.9, seed=2)
        t1 = srv.submit("square_root", gb, 0.5, seed=2)
        t2 = srv.submit("parallel_cc", gb, seed=2)
        assert srv.poll(t0)[0].cut == O.exact_mincut(ns, us, vs, ws)
        r = srv.poll(t1)[0]
        assert (r.cut, r.trials) == (want.cut, want.trials_per_rank)
        assert srv.poll(t2)[0].num_components == O.cc_labels(n, u, v)[0]


def test_over_budget_query_fails_alone(libcac):
    # K2500's root matrix (50 MB) exceeds a 32 MB budget: that query fails with CAC_ERR_OOM at
    # admission, reported in its own response; the queries around it are answered
    big = graphgen.complete(2500, 3)
    n, u, v, w = graphgen.erdos_renyi(150, 0.1, 4)
    with libcac.Server(0, hbm_budget_bytes=32 << 20) as srv:
        gb, gs = srv.graph(*big), srv.graph(n, u, v, w)
        t0 = srv.submit("square_root", gs, 0.9, seed=2)
        t1 = srv.submit("square_root", gb, 0.9, seed=2)
        t2 = srv.submit("square_root", gs, 0.9, seed=3)
        assert srv.poll(t0)[0].cut == O.exact_mincut(n, u, v, w)
        with pytest.raises(libcac.CacError) as e:
            srv.poll(t1)
        assert e.value.status == -2
        assert srv.poll(t2)[0].cut == O.exact_mincut(n, u, v, w)


def test_planned_levels_redone_in_the_serving_loop(libcac, ctx):
    # a complete graph with one dominant edge makes a planned level miss its target (a child's
    # round runs out of draws); the serving loop then runs every query in flight again level by
    # level, and every response still equals the single-query answer and the oracle's
    n, u, v, w = graphgen.complete(300, 1, wmax=1)
    w = np.asarray(w, np.uint32).copy()
    w[0] = 1000000
    specs = [(n, u, v, w), graphgen.erdos_renyi_m(1500, 12.0, 4, wmax=100),
             graphgen.watts_strogatz(300, 10, 0.3, 2, wmax=100)]
    singles = [ctx.graph(*s) for s in specs]
    qs = [(gi, sd) for sd in range(3) for gi in range(3)]
    expect = [(int(singles[gi].square_root(0.9, seed=sd).cut)) for gi, sd in qs]
    with libcac.Server(0) as srv:
        sg = [srv.graph(*s) for s in specs]
        tickets = [srv.submit("square_root", sg[gi], 0.9, seed=sd) for gi, sd in qs]
        got = [int(srv.poll(t)[0].cut) for t in tickets]
    assert got == expect
    for (gi, sd), c in zip(qs, got):
        sn, su, sv, sw = specs[gi]
        assert c == O.square_root(sn, su, sv, sw, 0.9, sd, ranks=1)[0]
