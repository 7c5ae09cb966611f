"""The batched uneven min-cut workload at full size: all 4096 graphs of the population (half
Watts-Strogatz, half G(n, M); n log-uniform in [64, 8192]; weights in [1, 100]; success
probability 0.9; seed = graph index) in one cac_mincut_batch, every cut compared with the exact
minimum cut of the same graph. The exact cuts come from the oracle's Nagamochi-Ono-Ibaraki
routine (the same value as Stoer-Wagner, the algorithm of the reference's base case
co_mincut_base_case.hpp:52-144; the two are compared in test_oracle_pins.py), run on every host
thread. Graphs are generated on the device; the oracle regenerates the same edges on the host
(graphgen, edge for edge identical, test_generate_gpu.py)."""
import os

import numpy as np
import pytest

import pyoracle as O
import workloads

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def test_every_batched_cut_is_exact(ctx):
    specs = workloads.uneven_population(4096)
    graphs = [workloads.make(ctx, sp) for sp in specs]
    try:
        seeds = [sp["seed"] for sp in specs]
        res = ctx.mincut_batch(graphs, 0.9, seeds=seeds)
        exact = O.exact_mincut_many([workloads.host_arrays(sp) for sp in specs], threads=os.cpu_count())
        got = np.array([int(r.cut) for r in res], dtype=np.uint64)
        want = np.array(exact, dtype=np.uint64)
        wrong = np.flatnonzero(got != want)
        assert wrong.size == 0, [(int(i), specs[i], int(got[i]), int(want[i])) for i in wrong[:5]]
        # the population spans the whole size range, the largest graphs included
        ns = np.array([g.n for g in graphs])
        assert ns.min() < 80 and ns.max() > 8000
        assert all(r.total_trials >= 1 for r in res)
    finally:
        for g in graphs:
            g.free()


def test_batch_of_the_largest_graphs_equals_one_by_one(ctx):
    # the 24 largest graphs of the population, batched and one by one: identical answers
    specs = workloads.uneven_population(4096)
    big = sorted(specs, key=lambda sp: -sp["n"])[:24]
    graphs = [workloads.make(ctx, sp) for sp in big]
    try:
        seeds = [sp["seed"] for sp in big]
        batch = ctx.mincut_batch(graphs, 0.9, seeds=seeds)
        for g, sd, r in zip(graphs, seeds, batch):
            alone = g.square_root(0.9, seed=sd)
            assert (r.cut, r.total_trials) == (alone.cut, alone.total_trials)
    finally:
        for g in graphs:
            g.free()
