"""Sparse Karger-Stein nodes (the reference's sparse recursion, co_mincut.h:131-155 and 401-405,
with WeightedIteratedSparseSampling::reduce's sort and merge, .cpp:26-234): nodes above the dense
limit, or above 2048 vertices with fewer than N^2 / 32 edges, stay edge lists; their children are
contracted by the Stage 1 rounds and relabelled, radix-sorted and merged on the device.

Every trial value equals the oracle's replay of the same counter stream, with the dense limit
lowered (cac_ctx_set_dense_limit / pyoracle.set_dense_limit) so that graphs of a few thousand
vertices take several sparse levels; at the default limit, plain Karger-Stein on more than 16384
vertices and square_root with a contracted size above 16384 run (they used to be refused) and
give the exact minimum cut."""
import numpy as np
import pytest

import cac
import graphgen
import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture
def lowered():
    """A context whose dense limit is 256 vertices, and the oracle set the same way."""
    c = cac.Context(0)
    c.set_dense_limit(256)
    O.set_dense_limit(256)
    yield c
    O.set_dense_limit(16384)
    c.close()


def _barbell(n, deg, bridges, seed):
    """Two G(n/2, M) halves with weights in [30, 100] joined by a few light edges (weights in
    [1, 20]): the minimum cut is the bridge bundle, far below every vertex's degree, so a trial
    finds it only through its contractions."""
    h = n // 2
    _, u1, v1, w1 = graphgen.erdos_renyi_m(h, deg, seed, wmax=100, wmin=30)
    _, u2, v2, w2 = graphgen.erdos_renyi_m(n - h, deg, seed + 1, wmax=100, wmin=30)
    rng = np.random.default_rng(seed)
    bu = rng.integers(0, h, bridges)
    bv = h + rng.integers(0, n - h, bridges)
    bw = rng.integers(1, 21, bridges)
    cat = lambda *xs: np.concatenate(xs).astype(np.uint32)  # noqa: E731
    return n, cat(u1, u2 + h, bu), cat(v1, v2 + h, bv), cat(w1, w2, bw)


def _ring(clusters, size, deg, seed):
    """Clusters (G(size, M), weights in [30, 100]) in a ring, neighbours joined by two light edges:
    many near-minimum cuts (any two bridge bundles)."""
    rng = np.random.default_rng(seed)
    us, vs, ws = [], [], []
    for c in range(clusters):
        _, u, v, w = graphgen.erdos_renyi_m(size, deg, seed + c, wmax=100, wmin=30)
        us.append(u + c * size)
        vs.append(v + c * size)
        ws.append(w)
        nxt = (c + 1) % clusters
        for _ in range(2):
            us.append([c * size + rng.integers(size)])
            vs.append([nxt * size + rng.integers(size)])
            ws.append([rng.integers(5, 25)])
    cat = lambda xs: np.concatenate([np.asarray(x) for x in xs]).astype(np.uint32)  # noqa: E731
    return clusters * size, cat(us), cat(vs), cat(ws)


@pytest.mark.parametrize("which", ["barbell", "ring", "er_unit"])
def test_karger_stein_sparse_trials_equal_replay(lowered, which):
    if which == "barbell":
        n, u, v, w = _barbell(1100, 10, 3, 12)
    elif which == "ring":
        n, u, v, w = _ring(6, 250, 12, 31)
    else:
        n, u, v, w = graphgen.erdos_renyi_m(700, 5.0, 13, wmax=1)
    assert 32 * len(u) < n * n  # a sparse root, several sparse levels under the lowered limit
    g = lowered.graph(n, u, v, w)
    got = g.karger_stein_trials(seed=5, trials=4)
    want = [O.ks_trial(n, u, v, w, 5, i) for i in range(4)]
    assert [int(x) for x in got] == want
    assert min(want) == O.exact_mincut(n, u, v, w)


def test_square_root_sparse_root_trials_equal_replay(lowered):
    # t = ceil(2 sqrt(m) + 1) above the lowered limit: Stage 1, then the contracted graph merged
    # by the device sort into a sparse root
    n, u, v, w = _barbell(5000, 14, 5, 21)
    t = O.intermediate_size(n, len(u))
    assert 256 < t < n
    g = lowered.graph(n, u, v, w)
    got = g.trials(seed=3, virtual_ranks=2, trials_per_rank=3)
    want = [[O.mincut_trial(n, u, v, w, 3, r, i) for i in range(3)] for r in range(2)]
    assert got.tolist() == want


def test_dense_graph_stays_dense_under_the_rule(lowered):
    # a dense root (32 m >= n^2) below the limit keeps the dense recursion: same values as before
    n, u, v, w = graphgen.erdos_renyi(200, 0.3, 31)
    assert 32 * len(u) >= n * n
    g = lowered.graph(n, u, v, w)
    got = g.karger_stein_trials(seed=1, trials=2)
    assert [int(x) for x in got] == [O.ks_trial(n, u, v, w, 1, i) for i in range(2)]


def test_karger_stein_above_16384_vertices_is_exact(ctx):
    # plain Karger-Stein on 20,000 vertices: the sparse levels, then dense nodes (default limit)
    n, u, v, w = graphgen.watts_strogatz(20000, 10, 0.4, 41, wmax=100)
    g = ctx.graph(n, u, v, w)
    res = g.karger_stein(0.9, seed=0)
    assert res.total_trials == O.ks_number_of_trials(n, 0.9)
    assert int(res.cut) == O.exact_mincut_noi(n, u, v, w)
    g.free()


def test_square_root_contracted_above_16384(ctx):
    # m > 6.7e7 edges, so t = ceil(2 sqrt(m) + 1) > 16384 < n: Stage 1 in global memory, each
    # trial's contracted graph sorted and merged into a sparse root of t vertices, dense children
    g = ctx.generate("erdos_renyi", seed=7, n=17500, p=0.45, wmin=1, wmax=42)
    t = O.intermediate_size(g.n, g.m)
    assert 16384 < t < g.n
    res = g.square_root(0.95, seed=0)
    assert res.intermediate == t and res.total_trials == O.number_of_trials(g.n, g.m, 0.95)
    u, v, w = g.edges()
    deg = np.bincount(u, weights=w, minlength=g.n) + np.bincount(v, weights=w, minlength=g.n)
    assert int(res.cut) == int(deg.min())  # a dense random graph: the minimum cut is a vertex's
    trial = g.trials(seed=0, virtual_ranks=1, trials_per_rank=2)[0]
    assert all(int(deg.min()) <= int(x) < 2 ** 63 for x in trial)  # every trial a real cut
    g.free()


def test_sparse_trials_with_u64_weights(lowered):
    # total weight above 2^32: the sparse lists carry u64 weights and the dense children u64
    # entries; every trial value still equals the replay
    n, u, v, _ = _barbell(900, 10, 3, 51)
    w = graphgen.weights(52, len(u), 1 << 22, 1 << 20)
    assert int(w.astype(np.uint64).sum()) >= 2 ** 32
    g = lowered.graph(n, u, v, w)
    got = g.karger_stein_trials(seed=2, trials=2)
    assert [int(x) for x in got] == [O.ks_trial(n, u, v, w, 2, i) for i in range(2)]
