"""Seeded graph populations and query traces of the batched and served min-cut workloads.

uneven_population   4096 independent graphs for one square_root batch: half Watts-Strogatz
                    (k even in [6, 32], rewiring 0.4), half Erdos-Renyi G(n, M) with average
                    degree uniform in [8, 64]; n log-uniform in [64, 8192]; weights in [1, 100];
                    success probability 0.9; seed = base + graph index.
served_population   graphs of a served stream: edge counts log-uniform in [10^3, 10^7],
                    alternately Erdos-Renyi G(n, p) and R-MAT (a=0.57, b=0.19, c=0.19), weights
                    in [1, 42]. The vertex count is chosen as floor(2 sqrt(m)) (R-MAT: the power
                    of two at or below it) so that square_root's pre-contraction target
                    ceil(2 sqrt(m) + 1) is at least n: the query is then the Karger-Stein budget on
                    the whole graph (a handful of trials). A sparse graph with 10^7 edges instead
                    needs 10^5 - 10^6 trials in any implementation of the reference's trial
                    budget, which no served query can afford.
served_trace        Poisson arrivals of square_root : approx_cut : parallel_cc queries in ratio
                    2:1:1 over a population, each with its own seed.

Specs are plain dicts understood by `make` (device generation through cac.Context.generate).
"""
import math

import numpy as np


def uneven_population(count=4096, base_seed=0):
    rng = np.random.default_rng(base_seed)
    specs = []
    for i in range(count):
        n = int(math.exp(rng.uniform(math.log(64), math.log(8192))))
        if i % 2 == 0:
            k = 2 * int(rng.integers(3, 17))  # even, 6 .. 32
            specs.append({"family": "watts_strogatz", "n": n, "k": k, "p": 0.4, "seed": base_seed + i,
                          "wmin": 1, "wmax": 100})
        else:
            deg = float(rng.uniform(8, 64))
            specs.append({"family": "erdos_renyi_m", "n": n, "avg_degree": deg, "seed": base_seed + i,
                          "wmin": 1, "wmax": 100})
    return specs


def served_population(count=32, base_seed=1000, m_lo=1e3, m_hi=1e7):
    rng = np.random.default_rng(base_seed)
    specs = []
    for i in range(count):
        m = math.exp(rng.uniform(math.log(m_lo), math.log(m_hi)))
        if i % 2 == 0:
            n = max(4, int(2 * math.sqrt(m)))
            p = min(1.0, m / (n * (n - 1) / 2))
            specs.append({"family": "erdos_renyi", "n": n, "p": p, "seed": base_seed + i, "wmin": 1, "wmax": 42})
        else:
            scale = max(2, int(math.floor(math.log2(2 * math.sqrt(m)))))
            ef = max(1, int(round(m / (1 << scale))))
            specs.append({"family": "rmat", "scale": scale, "edge_factor": ef, "seed": base_seed + i,
                          "wmin": 1, "wmax": 42})
    return specs


def served_trace(count, num_graphs, rate_per_s, seed=7):
    """-> list of (arrival_s, kind, graph_index, query_seed); rate_per_s = None: all at t = 0."""
    rng = np.random.default_rng(seed)
    kinds = ["square_root", "square_root", "approx_cut", "parallel_cc"]
    t = 0.0
    out = []
    for _ in range(count):
        if rate_per_s:
            t += float(rng.exponential(1.0 / rate_per_s))
        out.append((t, kinds[int(rng.integers(4))], int(rng.integers(num_graphs)), int(rng.integers(1 << 16))))
    return out


def make(ctx, spec):
    """Generate one spec on the device of `ctx` (a cac.Context)."""
    s = dict(spec)
    return ctx.generate(s.pop("family"), **s)


def host_arrays(spec):
    """The same graph from the host generators (graphgen) -> (n, u, v, w)."""
    import graphgen
    s = dict(spec)
    f = s.pop("family")
    if f == "erdos_renyi":
        return graphgen.erdos_renyi(s["n"], s["p"], s["seed"], wmax=s["wmax"], wmin=s["wmin"])
    if f == "erdos_renyi_m":
        return graphgen.erdos_renyi_m(s["n"], s["avg_degree"], s["seed"], wmax=s["wmax"], wmin=s["wmin"])
    if f == "watts_strogatz":
        return graphgen.watts_strogatz(s["n"], s["k"], s["p"], s["seed"], wmax=s["wmax"], wmin=s["wmin"])
    if f == "rmat":
        return graphgen.rmat(s["scale"], s["edge_factor"], s["seed"], wmax=s["wmax"], wmin=s["wmin"])
    if f == "complete":
        return graphgen.complete(s["n"], s["seed"], wmax=s["wmax"], wmin=s["wmin"])
    raise ValueError(f)
