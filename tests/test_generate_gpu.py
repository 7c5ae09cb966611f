"""Device generators (cac_graph_generate): the same edge list, in the same order, with the same
weights as graphgen's host generators, for every family and edge cases of each."""
import numpy as np
import pytest

import graphgen

pytestmark = pytest.mark.gpu


def _same(g, ref):
    n, u, v, w = ref
    assert g.n == n and g.m == len(u)
    gu, gv, gw = g.edges()
    assert np.array_equal(gu, u) and np.array_equal(gv, v) and np.array_equal(gw, w)
    assert g.total_weight == int(w.astype(np.uint64).sum())


@pytest.mark.parametrize("n,p,seed,wmax", [(2, 1.0, 0, 42), (50, 0.0, 1, 42), (300, 0.05, 2, 42), (1000, 0.05, 0, 42),
                                           (777, 0.3, 5, 1), (129, 1.0, 3, 100)])
def test_erdos_renyi(ctx, n, p, seed, wmax):
    _same(ctx.generate("erdos_renyi", seed=seed, n=n, p=p, wmax=wmax), graphgen.erdos_renyi(n, p, seed, wmax=wmax))


@pytest.mark.parametrize("n,deg,seed", [(1, 4.0, 0), (2, 7.0, 1), (64, 8.0, 2), (5000, 23.7, 3), (8192, 64.0, 4)])
def test_erdos_renyi_m(ctx, n, deg, seed):
    _same(ctx.generate("erdos_renyi_m", seed=seed, n=n, avg_degree=deg, wmax=100),
          graphgen.erdos_renyi_m(n, deg, seed, wmax=100))


@pytest.mark.parametrize("n,k,p,seed", [(10, 2, 0.0, 0), (64, 6, 0.4, 1), (3001, 32, 0.4, 2), (500, 10, 1.0, 3)])
def test_watts_strogatz(ctx, n, k, p, seed):
    _same(ctx.generate("watts_strogatz", seed=seed, n=n, k=k, p=p, wmax=100),
          graphgen.watts_strogatz(n, k, p, seed, wmax=100))


@pytest.mark.parametrize("scale,ef,seed,wmax", [(1, 1, 0, 1), (10, 16, 1, 1), (16, 16, 2, 1), (12, 8, 3, 42)])
def test_rmat(ctx, scale, ef, seed, wmax):
    _same(ctx.generate("rmat", seed=seed, scale=scale, edge_factor=ef, wmax=wmax),
          graphgen.rmat(scale, ef, seed, wmax=wmax))


@pytest.mark.parametrize("n,seed", [(2, 0), (33, 1), (600, 2)])
def test_complete(ctx, n, seed):
    _same(ctx.generate("complete", seed=seed, n=n, wmax=42), graphgen.complete(n, seed, wmax=42))


def test_rejects_bad_specs(libcac, ctx):
    with pytest.raises(libcac.CacError):
        ctx.generate("watts_strogatz", n=10, k=3, p=0.1, wmax=10)  # odd k
    with pytest.raises(libcac.CacError):
        ctx.generate("rmat", scale=0, edge_factor=16)
    with pytest.raises(libcac.CacError):
        ctx.generate("erdos_renyi", n=100, p=1.5)
    with pytest.raises(libcac.CacError):
        ctx.generate("complete", n=10, wmin=5, wmax=2)


def test_generated_graph_feeds_the_queries(ctx):
    g = ctx.generate("erdos_renyi", seed=0, n=1000, p=0.05, wmax=42)
    h = ctx.graph(*graphgen.erdos_renyi(1000, 0.05, 0))
    assert g.square_root(0.95, seed=0, virtual_ranks=4).cut == h.square_root(0.95, seed=0, virtual_ranks=4).cut == 620
    c1, l1, _ = g.connected_components()
    c2, l2, _ = h.connected_components()
    assert c1 == c2 and np.array_equal(l1, l2)
