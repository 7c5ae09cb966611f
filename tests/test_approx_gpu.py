"""Parity of the CUDA approx_cut path with the oracle's replay of the same counter-addressed keep
tests, and the O(log n)-approximation bound against the exact cut."""
import pytest

import graphgen
import pyoracle as O
from conftest import make_graph

pytestmark = pytest.mark.gpu


def test_reference_test_inputs(golden, ctx):
    for name, r in golden("ref_test_inputs.json").items():
        if name.startswith("cc_"):
            continue
        g = ctx.graph(r["n"], r["u"], r["v"], r["w"])
        for seed, ranks in ((0, 1), (3, 2), (11, 4)):
            res = g.approx_cut(0.9, seed=seed, virtual_ranks=ranks)
            want, level = O.approx_cut(r["n"], r["u"], r["v"], r["w"], 0.9, seed, ranks)
            assert (res.cut, res.level) == (want, level)
            assert res.copies == O.approx_trials(0.9) == 4
            assert res.trials == res.copies * res.level


@pytest.mark.parametrize("idx", range(5))
def test_seeded_graphs(golden, ctx, idx):
    spec = golden("mincut_seeded.json")[idx]
    n, u, v, w = make_graph(spec)
    g = ctx.graph(n, u, v, w)
    for seed, ranks, p in ((0, 1, 0.9), (5, 3, 0.95)):
        res = g.approx_cut(p, seed=seed, virtual_ranks=ranks)
        want, level = O.approx_cut(n, u, v, w, p, seed, ranks)
        assert (res.cut, res.level) == (want, level)
        # an O(log n) estimate: never far above the true cut
        assert res.cut <= 4 * spec["exact_cut"]


def test_fewer_edges_than_ranks(ctx):
    n, u, v, w = 3, [0, 1], [1, 2], [50, 60]
    g = ctx.graph(n, u, v, w)
    res = g.approx_cut(0.9, seed=1, virtual_ranks=5)
    assert (res.cut, res.level) == O.approx_cut(n, u, v, w, 0.9, 1, 5)


def test_larger_graph(ctx):
    n, u, v, w = graphgen.erdos_renyi_m(20000, 16, 3, wmax=42)
    g = ctx.graph(n, u, v, w)
    res = g.approx_cut(0.9, seed=2)
    assert (res.cut, res.level) == O.approx_cut(n, u, v, w, 0.9, 2, 1)


@pytest.mark.parametrize("ranks", [1, 3, 7])
def test_quad_path_large_graph(ctx, ranks):
    # more than 2^16 quads of 4 edges: one sitmo block per quad, hooks in slices; the same keep
    # decisions as the oracle's per-edge draws, so the same level, on 1 and several virtual ranks
    # (slices of m / P edges, the last with the rest)
    n, u, v, w = graphgen.erdos_renyi_m(15000, 40.0, 8, wmax=42)  # six or seven levels
    u, v, w = u[:-5], v[:-5], w[:-5]  # m not a multiple of 4 or of the rank count
    assert len(u) // 4 >= (1 << 16)
    g = ctx.graph(n, u, v, w)
    for seed in (0, 6):
        res = g.approx_cut(0.9, seed=seed, virtual_ranks=ranks)
        assert (res.cut, res.level) == O.approx_cut(n, u, v, w, 0.9, seed, ranks)


# ---- seed replay: the reference's own draws (cac_approx_cut_seed_replay) ----

def _approx_stream_graph(spec):
    import numpy as np
    n, u, v, w = make_graph(spec)
    if spec.get("unit"):
        w = np.ones_like(u)
    return n, u, v, w


def test_seed_replay_equals_reference_executable(golden, ctx):
    """The answers of the reference's approx_cut executable (one rank), seed by seed, on the
    unit-weight graphs of approx_stream.json."""
    runs = [r for r in golden("approx_stream.json")["runs"] if r.get("unit")]
    assert len(runs) == 5
    for spec in runs:
        n, u, v, w = _approx_stream_graph(spec)
        g = ctx.graph(n, u, v, w)
        got = [g.approx_cut(spec["success_probability"], seed=sd, seed_replay=True).cut for sd in spec["seeds"]]
        assert got == spec["weights"], spec["name"]


@pytest.mark.parametrize("ranks", [2, 3, 4])
def test_seed_replay_ranks_match_oracle(golden, ctx, ranks):
    """Several virtual ranks: slice r draws from sitmo(seed + r) at the reference's positions
    (levels after the first start at odd outputs: the CC seed takes one per level)."""
    for spec in [r for r in golden("approx_stream.json")["runs"] if r.get("unit")]:
        n, u, v, w = _approx_stream_graph(spec)
        g = ctx.graph(n, u, v, w)
        for sd in (0, 3, 9):
            res = g.approx_cut(0.9, seed=sd, virtual_ranks=ranks, seed_replay=True)
            assert (res.cut, res.level) == O.approx_cut_stream(n, u, v, w, 0.9, sd, ranks), (spec["name"], sd)


@pytest.mark.parametrize("ranks", [1, 3])
def test_seed_replay_large_graph(ctx, ranks):
    """More than 2^16 quads (hooks in slices), m not a multiple of 4 or of the rank count."""
    import numpy as np
    n, u, v, _ = graphgen.erdos_renyi_m(12000, 48.0, 17, wmax=1)
    u, v = u[:-3], v[:-3]
    w = np.ones_like(u)
    assert len(u) // 4 >= (1 << 16)
    g = ctx.graph(n, u, v, w)
    for sd in (0, 5):
        res = g.approx_cut(0.95, seed=sd, virtual_ranks=ranks, seed_replay=True)
        want = O.approx_cut_stream(n, u, v, w, 0.95, sd, ranks)
        assert (res.cut, res.level) == want and res.level >= 2  # levels after the first start at odd outputs


def test_seed_replay_refuses_weighted_graphs(ctx, libcac):
    import cac
    g = ctx.graph(3, [0, 1], [1, 2], [1, 2])
    with pytest.raises(cac.CacError, match="weight"):
        g.approx_cut(0.9, seed=0, seed_replay=True)


def test_level_count_follows_rank_slices(ctx):
    """ceil(ln w_r) of each rank's own slice, the smallest over ranks (ApproximateCut.cpp:19-30)."""
    n, u, v, w = 4, [0, 1, 2, 0], [1, 2, 3, 3], [1, 1, 1, 100]
    g = ctx.graph(n, u, v, w)
    res = g.approx_cut(0.9, seed=0, virtual_ranks=4)
    assert (res.cut, res.level) == (1, 0) == O.approx_cut(n, u, v, w, 0.9, 0, 4)
    res = g.approx_cut(0.9, seed=0, virtual_ranks=2)  # slices of weight 2 and 101: one level
    assert (res.cut, res.level) == O.approx_cut(n, u, v, w, 0.9, 0, 2)


def test_more_ranks_than_edges(ctx):
    """Every slice but the last is empty: no level runs (ceil(ln 0) levels on those ranks), in both
    modes, however many ranks are asked for."""
    n, u, v = 5, [0, 1, 2, 3], [1, 2, 3, 4]
    g = ctx.graph(n, u, v, [1, 1, 1, 1])
    for ranks in (5, 1 << 31):
        for replay in (False, True):
            res = g.approx_cut(0.9, seed=3, virtual_ranks=ranks, seed_replay=replay)
            assert (res.cut, res.level) == (1, 0)
    assert O.approx_cut(n, u, v, [1, 1, 1, 1], 0.9, 3, 5) == (1, 0)
