"""Many square_root queries of uneven graphs in one engine run (cac_mincut_batch): every result equals
the same query run alone, and the exact cut (Watts-Strogatz and G(n, M) graphs of uneven sizes, the
shape of the 4096-graph batch workload, at test size)."""
import numpy as np
import pytest

import graphgen
import pyoracle as O

pytestmark = pytest.mark.gpu


def _uneven_graphs(count, seed=100):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(64), np.log(600))))
        deg = float(rng.uniform(8, 24))
        if i % 2 == 0:
            k = max(6, 2 * int(deg // 2))
            out.append(graphgen.watts_strogatz(n, k, 0.4, seed + i, wmax=100))
        else:
            out.append(graphgen.erdos_renyi_m(n, deg, seed + i, wmax=100))
    return out


def test_batch_equals_one_by_one_and_exact(ctx):
    specs = _uneven_graphs(10)
    graphs = [ctx.graph(n, u, v, w) for n, u, v, w in specs]
    seeds = list(range(len(graphs)))
    batch = ctx.mincut_batch(graphs, 0.9, seeds=seeds, virtual_ranks=2)
    for (n, u, v, w), g, r, sd in zip(specs, graphs, batch, seeds):
        alone = g.square_root(0.9, seed=sd, virtual_ranks=2)
        assert r.cut == alone.cut
        assert r.total_trials == alone.total_trials and r.trials_per_rank == alone.trials_per_rank
        assert r.cut == O.exact_mincut(n, u, v, w)


def test_batch_per_trial_values_unchanged(ctx):
    # the same graph twice in one batch with different seeds: each equals its own replay
    n, u, v, w = graphgen.erdos_renyi(200, 0.08, 11)
    g = ctx.graph(n, u, v, w)
    r = ctx.mincut_batch([g, g], 0.95, seeds=[3, 4], virtual_ranks=1)
    for res, sd in zip(r, (3, 4)):
        per = res.trials_per_rank
        vals = [O.mincut_trial(n, u, v, w, sd, 0, i) for i in range(per)]
        assert res.cut == min(vals)


def test_empty_batch(ctx):
    assert ctx.mincut_batch([], 0.9) == []


def test_batch_mixes_entry_widths(ctx):
    # graphs whose total weight is at or above 2^32 keep u64 matrix entries, the others u32; one
    # batch holds both kinds in the same engine steps, and every answer is the exact cut
    light = [graphgen.erdos_renyi(150, 0.1, 21), graphgen.watts_strogatz(300, 8, 0.3, 22, wmax=100)]
    heavy = []
    for seed in (23, 24):
        n, u, v, _ = graphgen.erdos_renyi(140, 0.12, seed)
        w = graphgen.weights(seed, len(u), 2**31, 2**30)  # total weight far above 2^32
        heavy.append((n, u, v, w))
    specs = [light[0], heavy[0], light[1], heavy[1]]
    assert sum(int(w.astype(np.uint64).sum()) >= 2**32 for _, _, _, w in specs) == 2
    graphs = [ctx.graph(*sp) for sp in specs]
    res = ctx.mincut_batch(graphs, 0.9, seeds=[5, 6, 7, 8])
    for sp, g, r, sd in zip(specs, graphs, res, [5, 6, 7, 8]):
        assert r.cut == O.exact_mincut(*sp)
        assert r.cut == g.square_root(0.9, seed=sd).cut
