"""The oracle (CPU restatement) pinned against outputs of the reference itself."""
import numpy as np
import pytest

import pyoracle as O
from conftest import digest, make_graph


def _kat_cases(text):
    for line in text.strip().splitlines():
        head, vals = line.split(":")
        parts = head.split()
        yield parts[1], [int(x) for x in parts[2:6]], [int(x) for x in parts[6:10]], [int(x) for x in vals.split()]


def test_sitmo_matches_reference_engine(golden):
    cases = list(_kat_cases(golden("sitmo_kat.txt")))
    assert len(cases) == 28
    for kind, key, ctr, vals in cases:
        assert list(O.sitmo_outputs(key, ctr, len(vals))) == vals, (kind, key, ctr)
        if kind == "seed":
            assert [O.__dict__["lib"]().orc_sitmo_seed_output(key[0], k) for k in range(len(vals))] == vals


def test_draw64_is_word_of_block():
    key = [5, 7, 9, 0]
    blk = O.sitmo_block(key, [3, 2, 0, 0])
    for j in range(4):
        assert O.draw64(key, 2, 12 + j) == int(blk[j])


def test_cc_labels_match_reference_test_inputs(golden):
    ref = golden("ref_test_inputs.json")
    for name in ("cc_8.graph", "cc_13.graph"):
        r = ref[name]
        count, lab = O.cc_labels(r["n"], r["u"], r["v"])
        assert count == r["cc_count"] == r["parallel_cc_csv_count"] == 5
        assert lab.tolist() == r["cc_labels"]
        c2, lab2, _ = O.cc_iss(r["n"], r["u"], r["v"], 0)
        assert c2 == count and lab2.tolist() == r["cc_labels"]


@pytest.mark.parametrize("idx", range(5))
def test_cc_labels_match_reference_seeded(golden, idx):
    spec = golden("cc_seeded.json")[idx]
    n, u, v, w = make_graph(spec)
    assert digest(np.concatenate([u, v])) == spec["edges_sha256"]
    count, lab = O.cc_labels(n, u, v)
    assert count == spec["cc_count"]
    assert digest(lab) == spec["labels_sha256"]
    for ranks in (1, 3):
        c2, lab2, _ = O.cc_iss(n, u, v, spec["seed"], ranks)
        assert c2 == count and np.array_equal(lab2, lab)


def test_exact_cut_matches_reference(golden):
    ref = golden("ref_test_inputs.json")
    for name, r in ref.items():
        if name.startswith("cc_"):
            continue
        assert O.exact_mincut(r["n"], r["u"], r["v"], r["w"]) == r["exact_cut"] == r["square_root_cut"]


@pytest.mark.parametrize("idx", range(5))
def test_exact_and_square_root_oracle_match_reference_seeded(golden, idx):
    spec = golden("mincut_seeded.json")[idx]
    n, u, v, w = make_graph(spec)
    assert digest(np.concatenate([u, v, w])) == spec["edges_sha256"]
    assert O.exact_mincut(n, u, v, w) == spec["exact_cut"]
    assert O.number_of_trials(n, len(u), 0.95) == spec["square_root_trials"]
    if n <= 500:
        cut, per = O.square_root(n, u, v, w, 0.95, 0, 1)
        assert per == spec["square_root_trials"]
        assert cut == spec["exact_cut"]


def test_sparse_and_dense_stoer_wagner_agree():
    import graphgen
    for seed in range(3):
        n, u, v, w = graphgen.erdos_renyi_m(1100, 6, seed, wmax=9)
        dense_n, du, dv, dw = 300, u[(u < 300) & (v < 300)], v[(u < 300) & (v < 300)], w[(u < 300) & (v < 300)]
        # dense path (n <= 1024) vs the heap path on a relabelled copy forced above 1024 vertices
        a = O.exact_mincut(dense_n, du, dv, dw)
        big_n = 1500
        b = O.exact_mincut(big_n, du, dv, dw)  # vertices >= 300 isolated -> cut 0 on the big graph
        assert b == 0
        assert a == O.exact_mincut(dense_n, du, dv, dw)
    n, u, v, w = graphgen.erdos_renyi_m(1200, 12, 7, wmax=5)
    lab_count, _ = O.cc_labels(n, u, v)
    if lab_count == 1:
        mat = np.zeros((n, n), np.uint64)
        np.add.at(mat, (u, v), w.astype(np.uint64))
        np.add.at(mat, (v, u), w.astype(np.uint64))
        assert O.exact_mincut(n, u, v, w) == O.stoer_wagner_dense(mat)


def test_noi_exact_cut_equals_stoer_wagner(golden):
    # the Nagamochi-Ono-Ibaraki routine (used for thousands of graphs at a time) against the
    # Stoer-Wagner routines on the reference-pinned graphs, on random graphs of every family and
    # weight range (including disconnected ones, cut 0), and on graphs of the batched population
    import graphgen
    import workloads
    for name, r in golden("ref_test_inputs.json").items():
        if "exact_cut" in r:
            assert O.exact_mincut_noi(r["n"], r["u"], r["v"], r["w"]) == r["exact_cut"], name
    for spec in golden("mincut_seeded.json"):
        n, u, v, w = make_graph(spec)
        assert O.exact_mincut_noi(n, u, v, w) == spec["exact_cut"]
    for i in range(120):
        rng = np.random.default_rng(i)
        n = int(rng.integers(3, 300))
        kind = i % 4
        if kind == 0:
            g = graphgen.erdos_renyi(n, float(rng.uniform(0.01, 0.3)), i, wmax=int(rng.integers(1, 100)))
        elif kind == 1:
            g = graphgen.watts_strogatz(max(n, 12), 6, 0.4, i, wmax=100)
        elif kind == 2:
            g = graphgen.erdos_renyi_m(n, float(rng.uniform(1, 10)), i, wmax=5)
        else:
            g = graphgen.erdos_renyi(n, 0.02, i, wmax=1)
        assert O.exact_mincut_noi(*g) == O.exact_mincut(*g), i
    specs = workloads.uneven_population(4096)
    for sp in [s for s in specs if 1100 < s["n"] < 1600][:4]:
        g = workloads.host_arrays(sp)
        assert O.exact_mincut_noi(*g) == O.exact_mincut(*g), sp


def test_trial_values_are_upper_bounds_and_reach_the_cut(golden):
    spec = golden("mincut_seeded.json")[0]
    n, u, v, w = make_graph(spec)
    vals = [O.mincut_trial(n, u, v, w, 0, r, i) for r in range(2) for i in range(4)]
    assert min(vals) == spec["exact_cut"]
    assert all(x >= spec["exact_cut"] for x in vals)


def test_trial_budget_expressions():
    # co_mincut.cpp:18-41 and SquareRootCut.cpp:63-83 at the shapes of the benchmark configs
    assert O.ks_target(4000) == 2830 and O.ks_target(318) == 226 and O.ks_target(161) == 128
    assert O.intermediate_size(1000, 24910) == 317
    assert O.intermediate_size(4000, 7998000) == 4000
    assert O.number_of_trials(4000, 7998000, 0.95) == 7


def test_approx_threshold_matches_probability():
    for level in (1, 2, 5, 10):
        for w in (1, 2, 7, 42, 1000):
            f = O.keep_threshold(level, w) / 2.0**64
            assert abs(f - (1 - 2.0**-level) ** w) < 1e-12 * max(1, w)
    assert O.approx_trials(0.9) == 4


def test_approx_oracle_is_a_power_of_two_bound(golden):
    ref = golden("ref_test_inputs.json")
    for name, r in ref.items():
        if name.startswith("cc_"):
            continue
        cut, level = O.approx_cut(r["n"], r["u"], r["v"], r["w"], 0.9, 0)
        assert cut == 1 << level
        assert cut <= 2 * r["exact_cut"]


def test_ks_trial_count_matches_reference(golden):
    # comincut::number_of_trials (co_mincut.cpp:44-73), printed by the reference's own function
    for r in golden("ks_trials.json"):
        assert O.ks_number_of_trials(r["n"], r["p"]) == r["trials"], r


def test_karger_stein_oracle_matches_reference(golden):
    # the karger_stein executable's answers (src/executables/karger_stein.cpp, seed 0, p = 0.90)
    for name, r in golden("ref_test_inputs.json").items():
        if not name.startswith("cc_"):
            assert O.karger_stein(r["n"], r["u"], r["v"], r["w"], 0.9, 0)[0] == r["karger_stein_cut"], name
    for spec in golden("mincut_seeded.json"):
        if spec["n"] <= 500:
            n, u, v, w = make_graph(spec)
            cut, trials = O.karger_stein(n, u, v, w, 0.9, 0)
            assert trials == O.ks_number_of_trials(n, 0.9)
            assert cut == spec["karger_stein_cut"] == spec["exact_cut"], spec["name"]


def test_threaded_iss_restatement_equals_sequential():
    # the CPU baseline runs the reference's per-rank phases on one host thread per rank: the same
    # sample draws per rank, so the same rounds and labels as the sequential restatement
    import graphgen
    n, u, v, _ = graphgen.barabasi_albert(20000, 4, 3)
    want_count, want = O.cc_labels(n, u, v)
    for ranks in (1, 3, 8):
        c1, l1, r1 = O.cc_iss(n, u, v, 5, ranks, 1)
        c4, l4, r4 = O.cc_iss(n, u, v, 5, ranks, 4)
        assert (c1, r1) == (c4, r4) and c1 == want_count
        assert np.array_equal(l1, l4) and np.array_equal(l1, want)


def approx_graph(spec):
    """A graph of approx_stream.json, with unit weights where the spec says so."""
    n, u, v, w = make_graph(spec)
    if spec.get("unit"):
        w = np.ones_like(u)
    assert digest(np.concatenate([u, v, w])) == spec["edges_sha256"]
    return n, u, v, w


def test_binomial_stream_matches_libstdcxx(golden):
    """binomial_distribution<int>(w, 2^-level) on sitmo::prng_engine(seed), as the reference's
    approx_cut draws it: every draw and the engine position after them (its next raw output)."""
    cases = golden("approx_stream.json")["binomial"]
    assert len(cases) == 28
    for c in cases:
        got = O.ref_binomial_draws(c["seed"], c["level"], c["count"], c["weights"])
        assert got == (c["draws"], c["next_output"]), c


@pytest.mark.parametrize("idx", range(7))
def test_approx_stream_oracle_matches_reference_executable(golden, idx):
    """Every seed's answer of the reference's approx_cut executable (one rank) is reproduced by
    the replay of its own draws."""
    spec = golden("approx_stream.json")["runs"][idx]
    n, u, v, w = approx_graph(spec)
    got = [O.approx_cut_stream(n, u, v, w, spec["success_probability"], sd)[0] for sd in spec["seeds"]]
    assert got == spec["weights"]


def test_approx_level_count_follows_rank_slices():
    """The level count is ceil(ln w_r) of each rank's own slice (ApproximateCut.cpp:19-30), the
    smallest over ranks: a slice of weight 1 allows no level, so the answer is 2^0."""
    n = 4
    u = np.array([0, 1, 2, 0], dtype=np.uint32)
    v = np.array([1, 2, 3, 3], dtype=np.uint32)
    w = np.array([1, 1, 1, 100], dtype=np.uint32)  # slices of 4 ranks: weights 1, 1, 1, 100
    assert O.approx_cut(n, u, v, w, 0.9, 0, 4) == (1, 0)
    assert O.approx_cut_stream(n, u, v, w, 0.9, 0, 4) == (1, 0)
    # one rank: ceil(ln 103) = 5 levels; the cycle's cut (2) disconnects by level 5
    assert O.approx_cut(n, u, v, w, 0.9, 0, 1)[1] >= 1


def test_group_variant_layout_and_answer():
    """SquareRootCut's group variant (SquareRootCut.cpp:188-298): with p >= 2T ranks the groups
    have the largest power-of-two size not above p / T (integer division), p / size groups in
    all, one trial each; Stage 1 draws floor(n0^(1 + 0.1 / 2)) edges per round in float
    (WeightedIteratedSparseSampling.hpp:66-67). The answer is the smallest group value (or the
    minimum weighted degree), which is the exact cut on these graphs."""
    assert [O.group_count(p, t) for p, t in [(24, 6), (100, 7), (12, 6), (13, 6), (1024, 3)]] == [6, 12, 6, 6, 4]
    assert [O.group_draws(n) for n in (2, 100, 1000, 4096)] == [int(np.float32(n) ** np.float32(1.05))
                                                               for n in (2, 100, 1000, 4096)]
    n, u, v, w = make_graph({"kind": "er", "n": 120, "p": 0.15, "seed": 5, "wmax": 30})
    T = O.number_of_trials(n, len(u), 0.9)
    cut, per = O.square_root(n, u, v, w, 0.9, 2, ranks=2 * T)
    groups = [O.mincut_group_trial(n, u, v, w, 2, g) for g in range(O.group_count(2 * T, T))]
    assert per == 1 and cut <= min(groups) and cut == O.exact_mincut_noi(n, u, v, w)
