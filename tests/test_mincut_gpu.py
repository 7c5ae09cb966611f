"""Parity of the CUDA min-cut path (square_root) with the oracle, through the C ABI.

Three tiers:
  * kernel level: the Stoer-Wagner leaf kernel against the oracle's exact cut, one dense
    Karger-Stein trial against the oracle's replay of the same counter-addressed trial;
  * trial level: every trial value equal to the oracle's CPU replay of that trial, bit for bit;
  * result level: the square_root answer equal to the exact minimum cut (Stoer-Wagner) and to the
    reference's own square_root output on the pinned graphs.
"""
import numpy as np
import pytest

import graphgen
import pyoracle as O
from conftest import make_graph

pytestmark = pytest.mark.gpu


def _dense(n, u, v, w):
    mat = np.zeros((n, n), np.uint64)
    np.add.at(mat, (u, v), np.asarray(w, np.uint64))
    np.add.at(mat, (v, u), np.asarray(w, np.uint64))
    np.fill_diagonal(mat, 0)
    return mat


def _random_dense(n, seed, density=0.3, wmax=42, big=False):
    rng = np.random.default_rng(seed)
    mask = np.triu(rng.random((n, n)) < density, 1)
    w = rng.integers(1, wmax + 1, size=(n, n), dtype=np.uint64)
    if big:
        w = w << np.uint64(33)
    mat = np.where(mask, w, 0).astype(np.uint64)
    return mat + mat.T


@pytest.mark.parametrize("n,density,big", [(2, 1.0, False), (3, 0.7, False), (17, 0.4, False), (64, 0.2, False),
                                           (100, 0.05, False), (128, 0.3, False), (128, 0.02, False),
                                           (90, 0.3, True)])
def test_leaf_stoer_wagner_kernel(ctx, n, density, big):
    for seed in range(3):
        mat = _random_dense(n, seed, density, big=big)
        assert ctx.exact_cut_small(mat) == O.stoer_wagner_dense(mat)


# The leaf kernel keeps 32-bit keys packed with the vertex (one reduction per step) while the leaf
# weighs less than 2^24, 32-bit keys with a two-step argmax up to 2^32, 64-bit keys above: one
# case per form, on random leaves and on two dense clusters joined by a few light edges (the
# minimum cut is the bridge, below every degree, so orderings contract each cluster first and a
# second ordering finds the bridge).
def _two_clusters(n, seed, wmax, bridges=3):
    mat = _random_dense(n, seed, 0.6, wmax=wmax)
    h = n // 2
    mat[:h, h:] = 0
    mat[h:, :h] = 0
    rng = np.random.default_rng(seed + 1000)
    for _ in range(bridges):
        a, b = int(rng.integers(0, h)), int(rng.integers(h, n))
        mat[a, b] = mat[b, a] = mat[a, b] + 1
    return mat


@pytest.mark.parametrize("wmax", [42, 1 << 18, 1 << 40])
@pytest.mark.parametrize("n", [128, 77, 6])
def test_leaf_kernel_key_widths_and_clusters(ctx, n, wmax):
    for seed in range(3):
        mat = _random_dense(n, seed, 0.5, wmax=wmax)
        assert ctx.exact_cut_small(mat) == O.stoer_wagner_dense(mat)
        mat = _two_clusters(n, seed, wmax)
        got = ctx.exact_cut_small(mat)
        assert got == O.stoer_wagner_dense(mat)
        assert got <= 3


@pytest.mark.parametrize("n,density", [(129, 0.5), (200, 0.1), (318, 0.15), (500, 0.05)])
def test_dense_karger_stein_trial_matches_replay(ctx, n, density):
    mat = _random_dense(n, n, density)
    for seed, rank, trial in ((0, 0, 0), (5, 1, 3), (123, 3, 17)):
        assert ctx.ks_dense(mat, seed, rank, trial) == O.ks_dense(mat, seed, rank, trial)


def test_dense_karger_stein_disconnected(ctx):
    mat = _random_dense(300, 1, 0.2)
    mat[:150, 150:] = 0
    mat[150:, :150] = 0
    assert ctx.ks_dense(mat, 0, 0, 0) == 0 == O.ks_dense(mat, 0, 0, 0)


@pytest.mark.parametrize("idx", range(5))
def test_every_trial_matches_replay(golden, ctx, idx):
    spec = golden("mincut_seeded.json")[idx]
    n, u, v, w = make_graph(spec)
    g = ctx.graph(n, u, v, w)
    ranks, per = (2, 3) if n <= 500 else (1, 4)
    got = g.trials(seed=7, virtual_ranks=ranks, trials_per_rank=per)
    for r in range(ranks):
        for i in range(per):
            assert int(got[r, i]) == O.mincut_trial(n, u, v, w, 7, r, i), (r, i)
    assert got.min() >= spec["exact_cut"]


@pytest.mark.parametrize("idx", range(5))
def test_square_root_equals_exact_cut(golden, ctx, idx):
    spec = golden("mincut_seeded.json")[idx]
    n, u, v, w = make_graph(spec)
    g = ctx.graph(n, u, v, w)
    for ranks in (1, 4):
        res = g.square_root(0.95, seed=0, virtual_ranks=ranks)
        assert res.cut == spec["exact_cut"] == spec["square_root_cut"]
        assert res.trials_per_rank == -(-spec["square_root_trials"] // ranks)


def test_reference_known_answers(golden, ctx):
    for name, r in golden("ref_test_inputs.json").items():
        if name.startswith("cc_"):
            continue
        g = ctx.graph(r["n"], r["u"], r["v"], r["w"])
        assert g.square_root(0.95, seed=0).cut == r["exact_cut"] == r["square_root_cut"]


@pytest.mark.parametrize("case", ["single_edge", "disconnected", "isolated_vertex", "parallel_and_loops"])
def test_edge_cases(ctx, case):
    if case == "single_edge":
        n, u, v, w = 2, [0], [1], [9]
    elif case == "disconnected":
        n, u, v, w = graphgen.erdos_renyi(300, 0.1, 3)
        keep = (u < 150) == (v < 150)
        u, v, w = u[keep], v[keep], w[keep]
    elif case == "isolated_vertex":
        n, u, v, w = graphgen.erdos_renyi(200, 0.2, 4)
        keep = (u != 7) & (v != 7)
        u, v, w = u[keep], v[keep], w[keep]
    else:
        n, u, v, w = graphgen.erdos_renyi(150, 0.2, 5)
        u = np.concatenate([u, u[:50], np.arange(10, dtype=np.uint32)])
        v = np.concatenate([v, v[:50], np.arange(10, dtype=np.uint32)])
        w = np.concatenate([w, w[:50], np.full(10, 5, np.uint32)])
    u, v, w = (np.asarray(x, np.uint32) for x in (u, v, w))
    g = ctx.graph(n, u, v, w)
    want = O.exact_mincut(n, u, v, w)
    assert g.square_root(0.95, seed=1).cut == want
    got = g.trials(seed=2, virtual_ranks=1, trials_per_rank=3)
    for i in range(3):
        assert int(got[0, i]) == O.mincut_trial(n, u, v, w, 2, 0, i)


def test_rejects_single_vertex(ctx, libcac):
    g = ctx.graph(1, np.zeros(0, np.uint32), np.zeros(0, np.uint32))
    with pytest.raises(libcac.CacError) as e:
        g.square_root(0.95, 0)
    assert e.value.status == -1


# Stage 1 of graphs with more than 16384 vertices runs in global memory (shrink_big.cu); every
# trial still equals the oracle's replay of the same counter stream.
def _ring_plus_er(n, deg, seed):
    """A weighted ring (connected, no isolated vertex) plus G(n, M) edges."""
    _, u, v, w = graphgen.erdos_renyi_m(n, deg, seed, wmax=100)
    ring = np.arange(n, dtype=np.uint32)
    rw = graphgen.weights(seed + 1, n, 60, 20)
    return n, np.concatenate([ring, u]), np.concatenate([(ring + 1) % n, v]).astype(np.uint32), np.concatenate([rw, w])


@pytest.mark.parametrize("spec", [
    ("ring_er", 20000, 6.0, 3),  # t ~ 500: bisection of the last round's draws
    ("ring_er", 40000, 3.0, 4),  # sparser, more rounds
    ("ws", 17000, 4, 5),         # ring lattice, rewired: long paths
])
def test_large_graph_trials_match_replay(ctx, spec):
    if spec[0] == "ring_er":
        n, u, v, w = _ring_plus_er(spec[1], spec[2], spec[3])
    else:
        n, u, v, w = graphgen.watts_strogatz(spec[1], spec[2], 0.3, spec[3], wmax=100)
    g = ctx.graph(n, u, v, w)
    got = g.trials(seed=9, virtual_ranks=2, trials_per_rank=2)
    for r in range(2):
        for i in range(2):
            assert int(got[r, i]) == O.mincut_trial(n, u, v, w, 9, r, i), (spec, r, i)


def test_large_disconnected_graph_trials(ctx):
    # 30000 vertices, edges only among the first 2000: Stage 1 stops with every remaining edge a
    # loop and more than 16384 vertices left; the cut is 0, as in the replay
    n0, u, v, w = graphgen.erdos_renyi_m(2000, 10.0, 6, wmax=50)
    n = 30000
    g = ctx.graph(n, u, v, w)
    got = g.trials(seed=1, virtual_ranks=1, trials_per_rank=3)
    for i in range(3):
        assert int(got[0, i]) == O.mincut_trial(n, u, v, w, 1, 0, i) == 0
    assert g.square_root(0.5, seed=1).cut == 0


def test_click_graph_on_device(golden, libcac, ctx):
    # the device form of CLICK equals the host generator; square_root finds the exact cut that the
    # reference's exact Stoer-Wagner reports for the reference's own CLICK graph
    for case in golden("click.json"):
        if "exact_cut" not in case or case["n"] < 3:
            continue
        g = ctx.click(case["n"], case["ranks"], case["seed"])
        _, u, v, w = libcac.click_edges(case["n"], case["ranks"], case["seed"])
        gu, gv, gw = g.edges()
        assert np.array_equal(gu, u) and np.array_equal(gv, v) and np.array_equal(gw, w)
        assert g.square_root(0.95, seed=case["seed"]).cut == case["exact_cut"]


# Plain Karger-Stein on the whole graph (the reference's karger_stein executable,
# src/executables/karger_stein.cpp:34, comincut::minimum_cut with its own trial count): every
# answer equals the oracle's replay of the same trials from the full n x n matrix.
def _ks_cases(golden):
    for name, r in golden("ref_test_inputs.json").items():
        if not name.startswith("cc_"):
            yield name, (r["n"], np.asarray(r["u"], np.uint32), np.asarray(r["v"], np.uint32),
                         np.asarray(r["w"], np.uint32)), r["karger_stein_cut"]
    for spec in golden("mincut_seeded.json"):
        if spec["n"] <= 500:
            yield spec["name"], make_graph(spec), spec["karger_stein_cut"]
    yield "ws_700", graphgen.watts_strogatz(700, 8, 0.3, 21, wmax=100), None
    # total weight above 2^32: 64-bit node matrices
    yield "er_300_big", graphgen.erdos_renyi(300, 0.2, 22, wmin=1 << 24, wmax=1 << 26), None


def test_karger_stein_matches_replay_and_reference(golden, ctx):
    for name, (n, u, v, w), ref_cut in _ks_cases(golden):
        g = ctx.graph(n, u, v, w)
        for seed in (0, 9):
            r = g.karger_stein(0.9, seed)
            cut, trials = O.karger_stein(n, u, v, w, 0.9, seed)
            assert (int(r.cut), r.trials_per_rank, r.total_trials, r.intermediate) == (cut, trials, trials, n), name
            if seed == 0 and ref_cut is not None:
                assert cut == ref_cut


def test_karger_stein_probabilities_and_edges(ctx, libcac):
    n, u, v, w = graphgen.erdos_renyi(260, 0.1, 23)
    g = ctx.graph(n, u, v, w)
    for p in (0.0, 0.5, 0.99):
        r = g.karger_stein(p, 4)
        assert (int(r.cut), r.trials_per_rank) == O.karger_stein(n, u, v, w, p, 4)
    # two vertices, a disconnected graph
    assert ctx.graph(2, [0], [1], [9]).karger_stein(0.9, 0).cut == 9
    keep = (u < 130) == (v < 130)
    assert ctx.graph(n, u[keep], v[keep], w[keep]).karger_stein(0.9, 1).cut == 0
    for bad in (1.0, -0.1):
        with pytest.raises(libcac.CacError):
            g.karger_stein(bad, 0)
    with pytest.raises(libcac.CacError):
        ctx.graph(1, np.zeros(0, np.uint32), np.zeros(0, np.uint32)).karger_stein(0.9, 0)


def test_karger_stein_above_the_dense_limit_runs_sparse(ctx):
    # 20,000 vertices: the root and the first levels are edge lists (the reference's sparse
    # recursion), later levels dense; the answer is the exact cut
    n, u, v, w = _ring_plus_er(20000, 2, 24)
    res = ctx.graph(n, u, v, w).karger_stein(0.9, 0)
    assert res.total_trials == O.ks_number_of_trials(n, 0.9)
    assert int(res.cut) == O.exact_mincut_noi(n, u, v, w)


@pytest.mark.parametrize("big", [False, True])
def test_shared_row_quotient_trials_match_replay(ctx, big):
    # K2100 keeps t = n, so the first quotient steps have N >= 2000 and take the shared-row kernel
    # (8 warps on one output row); u32 node matrices, and u64 when the total weight passes 2^32
    n = 2100
    if big:
        n, u, v, w = graphgen.complete(n, 31, wmin=1 << 20, wmax=1 << 22)
    else:
        n, u, v, w = graphgen.complete(n, 31)
    assert O.intermediate_size(n, len(u)) >= n
    got = ctx.graph(n, u, v, w).trials(seed=5, virtual_ranks=1, trials_per_rank=2)
    for i in range(2):
        assert int(got[0, i]) == O.mincut_trial(n, u, v, w, 5, 0, i)


@pytest.mark.slow
def test_full_size_k4000_trials_match_replay(ctx):
    """The square_root configuration K4000 with weights in [1, 42] at full size: 7 trials, every
    trial value equal to the oracle's replay of the same counter stream (the trials replayed on
    host threads at once), and the answer is the minimum weighted degree."""
    from concurrent.futures import ThreadPoolExecutor
    n, u, v, w = graphgen.complete(4000, 0)
    assert len(u) == 7998000 and O.number_of_trials(n, len(u), 0.95) == 7
    g = ctx.graph(n, u, v, w)
    res = g.square_root(0.95, seed=0)
    got = g.trials(seed=0, virtual_ranks=1, trials_per_rank=7)[0]
    with ThreadPoolExecutor(max_workers=7) as pool:
        want = list(pool.map(lambda i: O.mincut_trial(n, u, v, w, 0, 0, i), range(7)))
    assert [int(x) for x in got] == want
    deg = np.zeros(n, np.uint64)
    np.add.at(deg, u, w.astype(np.uint64))
    np.add.at(deg, v, w.astype(np.uint64))
    assert res.total_trials == 7 and res.cut == min(want) == int(deg.min())


@pytest.mark.parametrize("kind", [1, 2, 3, 4])
@pytest.mark.parametrize("heavy", [False, True])
def test_every_quotient_kernel_matches_replay(libcac, kind, heavy):
    # the three quotient kernels (warp per row, eight warps per row, warp per row with member rows
    # staged by bulk copies) each forced for every step, and the size rule without timing: trial
    # values equal the replay, with u32 node matrices and with u64 ones (total weight above 2^32)
    c = libcac.Context(0)
    try:
        c.set_quotient_kernel(kind)
        if heavy:
            n, u, v, w = graphgen.erdos_renyi(700, 0.2, 41, wmin=1 << 20, wmax=1 << 22)
        else:
            n, u, v, w = graphgen.complete(1500, 42)
        got = c.graph(n, u, v, w).trials(seed=7, virtual_ranks=1, trials_per_rank=2)
        assert [int(x) for x in got[0]] == [O.mincut_trial(n, u, v, w, 7, 0, i) for i in range(2)]
    finally:
        c.close()


# Planning ahead (the default): the Karger-Stein levels of a run follow one another with every
# child taken at its target size, and a child that stops elsewhere sends the run back to the
# level-by-level schedule. Either way every trial equals the oracle's replay: on graphs whose
# children all reach their targets (no redo), on a complete graph with one dominant edge (rounds
# run out of draws: children are carried into another round, so the planned run is redone) and on
# a disconnected graph (sources without edges).
def _heavy_complete(n, seed):
    n, u, v, w = graphgen.complete(n, seed, wmax=1)
    w = np.asarray(w, np.uint32).copy()
    w[0] = 1000000
    return n, u, v, w


@pytest.mark.parametrize("case", ["er", "ws", "heavy", "disconnected"])
def test_plan_ahead_and_level_by_level_agree(libcac, case):
    if case == "er":
        n, u, v, w = graphgen.erdos_renyi(1000, 0.05, 0, wmax=42)
    elif case == "ws":
        n, u, v, w = graphgen.watts_strogatz(3000, 10, 0.3, 4, wmax=100)
    elif case == "heavy":
        n, u, v, w = _heavy_complete(300, 1)
    else:  # 200 disjoint triangles: Stage 1 stops at 200 isolated vertices, the root has no edges
        base = np.arange(200, dtype=np.uint32) * 3
        u = np.concatenate([base, base, base + 1])
        v = np.concatenate([base + 1, base + 2, base + 2])
        w = np.full(600, 7, np.uint32)
        n = 600
    got = {}
    redos = {}
    for plan in (True, False):
        c = libcac.Context(0)
        try:
            c.set_plan_ahead(plan)
            got[plan] = c.graph(n, u, v, w).trials(seed=3, virtual_ranks=2, trials_per_rank=2)
            redos[plan] = c.plan_redos()
        finally:
            c.close()
    assert np.array_equal(got[True], got[False])
    for r in range(2):
        for i in range(2):
            assert int(got[True][r, i]) == O.mincut_trial(n, u, v, w, 3, r, i), (case, r, i)
    assert redos[False] == 0
    if case in ("er", "ws"):
        assert redos[True] == 0
    else:
        assert redos[True] == 1
