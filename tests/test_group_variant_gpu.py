"""Parity of square_root's group variant (the reference's high-concurrency path,
SquareRootCut::participateInGroup, src/SquareRootCut.cpp:188-298) with the oracle.

With virtual_ranks >= 2T the ranks form groups of the largest power of two not above
virtual_ranks / T; each group runs one trial: Stage 1 in rounds of floor(n^1.05) weighted draws
(WeightedIteratedSparseSampling, .hpp:66-67) down to t vertices, then two Karger-Stein recursions
from the contracted graph. Every group's value equals the oracle's replay of the same counter
stream (pyoracle.mincut_group_trial), on dense roots, on the whole graph (t >= n), on graphs with
more than 16384 vertices and on sparse roots (t above the dense limit); the answer equals the
oracle's square_root in the same mode and the exact minimum cut."""
import numpy as np
import pytest

import cac
import graphgen
import pyoracle as O

pytestmark = pytest.mark.gpu


def _ring_plus_er(n, deg, seed):
    _, u, v, w = graphgen.erdos_renyi_m(n, deg, seed, wmax=100)
    ring = np.arange(n, dtype=np.uint32)
    rw = graphgen.weights(seed + 1, n, 60, 20)
    return n, np.concatenate([ring, u]), np.concatenate([(ring + 1) % n, v]).astype(np.uint32), np.concatenate([rw, w])


def _want(n, u, v, w, seed, groups):
    return [O.mincut_group_trial(n, u, v, w, seed, g) for g in range(groups)]


def test_layout_of_the_group_variant(ctx):
    n, u, v, w = graphgen.erdos_renyi_m(300, 20, 3, wmax=100)
    T = O.number_of_trials(n, len(u), 0.5)
    g = ctx.graph(n, u, v, w)
    for ranks in (2 * T - 1, 2 * T, 3 * T, 8 * T + 5, 64):
        res = g.square_root(0.5, seed=3, virtual_ranks=ranks)
        if ranks >= 2 * T:
            assert res.high_concurrency == 1
            assert res.trials_per_rank == 1
            assert res.total_trials == O.group_count(ranks, T)
        else:
            assert res.high_concurrency == 0
            assert res.total_trials == ranks * -(-T // ranks)
        assert (int(res.cut), res.trials_per_rank) == O.square_root(n, u, v, w, 0.5, 3, ranks=ranks)


@pytest.mark.parametrize("spec", [
    ("er", 300, 20, 3),      # t = 111 < n: Stage 1 rounds, dense root
    ("er", 1000, 8, 4),      # sparser: more rounds
    ("ws", 2500, 6, 5),      # long paths
    ("complete", 150, 0, 6), # t >= n: the recursions start from the whole graph
])
def test_every_group_matches_replay(ctx, spec):
    kind, n, deg, seed = spec
    if kind == "er":
        n, u, v, w = graphgen.erdos_renyi_m(n, deg, seed, wmax=100)
    elif kind == "ws":
        n, u, v, w = graphgen.watts_strogatz(n, deg, 0.3, seed, wmax=100)
    else:
        n, u, v, w = graphgen.complete(n, seed)
    got = ctx.graph(n, u, v, w).group_trials(seed=11, groups=6)
    assert [int(x) for x in got] == _want(n, u, v, w, 11, 6), spec


def test_groups_above_16384_vertices(ctx):
    n, u, v, w = _ring_plus_er(20000, 6, 7)
    got = ctx.graph(n, u, v, w).group_trials(seed=2, groups=3)
    assert [int(x) for x in got] == _want(n, u, v, w, 2, 3)


def test_disconnected_graph_groups_are_zero(ctx):
    n0, u, v, w = graphgen.erdos_renyi_m(2000, 10.0, 6, wmax=50)
    got = ctx.graph(30000, u, v, w).group_trials(seed=1, groups=2)
    assert [int(x) for x in got] == _want(30000, u, v, w, 1, 2) == [0, 0]


@pytest.fixture
def lowered():
    c = cac.Context(0)
    c.set_dense_limit(256)
    O.set_dense_limit(256)
    yield c
    O.set_dense_limit(16384)
    c.close()


@pytest.mark.parametrize("spec", [("er", 3000, 12, 8), ("ws", 5000, 10, 9)])
def test_sparse_roots_match_replay(lowered, spec):
    # t above the lowered dense limit: the contracted graph is a merged edge list shared by the
    # group's two recursions
    kind, n, deg, seed = spec
    if kind == "er":
        n, u, v, w = _ring_plus_er(n, deg, seed)
    else:
        n, u, v, w = graphgen.watts_strogatz(n, deg, 0.4, seed, wmax=100)
    assert O.intermediate_size(n, len(u)) > 256
    got = lowered.graph(n, u, v, w).group_trials(seed=4, groups=3)
    assert [int(x) for x in got] == _want(n, u, v, w, 4, 3), spec


def test_high_concurrency_answer_is_exact(ctx):
    for seed in range(3):
        n, u, v, w = graphgen.watts_strogatz(600, 6, 0.3, 20 + seed, wmax=100)
        T = O.number_of_trials(n, len(u), 0.9)
        res = ctx.graph(n, u, v, w).square_root(0.9, seed=seed, virtual_ranks=4 * T)
        assert res.high_concurrency == 1
        assert (int(res.cut), 1) == O.square_root(n, u, v, w, 0.9, seed, ranks=4 * T)
        assert int(res.cut) == O.exact_mincut_noi(n, u, v, w)


def test_batch_and_server_take_the_group_variant(ctx, libcac):
    specs = [graphgen.erdos_renyi_m(300, 20, s, wmax=100) for s in range(3)] + \
            [graphgen.watts_strogatz(800, 6, 0.3, 7, wmax=100)]
    graphs = [ctx.graph(*sp) for sp in specs]
    ranks = 200
    batch = ctx.mincut_batch(graphs, 0.5, seeds=[5, 6, 7, 8], virtual_ranks=ranks)
    for g, sp, sd, r in zip(graphs, specs, [5, 6, 7, 8], batch):
        alone = g.square_root(0.5, seed=sd, virtual_ranks=ranks)
        assert (r.cut, r.total_trials, r.high_concurrency) == (alone.cut, alone.total_trials, alone.high_concurrency)
        assert (int(r.cut), r.trials_per_rank) == O.square_root(*sp, 0.5, sd, ranks=ranks)
    srv = libcac.Server(0)
    try:
        sg = srv.graph(*specs[3])
        resp, _ = srv.poll(srv.submit("square_root", sg, 0.5, seed=8, virtual_ranks=ranks))
        assert (int(resp.cut), resp.trials) == (int(batch[3].cut), 1)
    finally:
        srv.close()
