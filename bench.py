"""Benchmark: parallel_cc connected components on the Barabasi-Albert graph with 1,024,000
vertices and attachment 16 (16,383,744 undirected edges, unweighted, uint32 ids, edge list
randomly permuted by seed 0) — the graph of the reference's own published CC measurement.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl cac|reference]

One step = one connected-components query over the whole graph (sampling round + closing edge
pass + labels), i.e. one call of UnweightedIteratedSparseSampling::connectedComponents in the
reference. The metric is edges per second.

  value      device-resident graph; CUDA events on the library's stream around each query; the
             L2 is flushed (a 512 MB write) before every timed query, outside the events.
  e2e        the same query through the one-call C ABI entry point from pinned HOST edge arrays
             to HOST labels, host->device and device->host copies inside the timed region.
  roofline   the whole query against HBM: algorithmic bytes 8 m + 8 n per query (u and v read
             once, parent initialised and label written once) / the query's CUDA-event
             duration, against the measured HBM copy bandwidth; the closing filter pass over all
             edges (8 m bytes per launch) is reported beside it as its own kernel roofline.
  cpu_baseline  the oracle's restatement of the reference's CC loop on the host with the same 16
                virtual ranks, each on its own thread (the reference under mpiexec -n 16).
  also_*     the other configurations of the metric: CC on R-MAT scale 22, square_root
             (Karger-Stein trials/s) on ER(1000, 0.05) and K4000, plain Karger-Stein on the
             32,000-vertex Watts-Strogatz shape of the reference's published karger_stein
             baseline (sparse recursion on top, dense below), 512 graphs of the uneven
             batched population (batched vs one call per graph, every cut checked against the
             exact cut), and a shortened served stream (queries/s, p50/p99).

Both arms run the query with 16 virtual ranks (the reference's mpiexec -n 16; CC labels do not
depend on the rank count).

--impl reference times the reference's CPU implementation of the path (the oracle port of
UnweightedIteratedSparseSampling::connectedComponents; the reference sources themselves are not
present on the GPU host) on the same workload and prints the same JSON line, with the port's
measured slowdown against the reference's own build beside it.

N > 1 (torchrun): every rank runs an independent replica of the query on its own GPU ("replicas
only": the reference's CC has no exchange that a single GPU would need); value = edges of all
ranks / max time over ranks.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import tempfile
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "comm-avoiding-cuts-cc_gb300")
sys.path.insert(0, PKG)

import numpy as np  # noqa: E402
from concurrent.futures import ThreadPoolExecutor  # noqa: E402

N_VERTICES, ATTACH, GRAPH_SEED = 1024000, 16, 0
VIRTUAL_RANKS = 16  # both arms: the reference under mpiexec -n 16
# The oracle port against the reference's own build, one core each, same machine and inputs
# (oracle/refbuild/port_speed.py, run where both exist): how much the port-based CPU baseline
# understates the reference.
_PORT_HOW = ("oracle/refbuild/port_speed.py: one core each of an Intel Xeon @ 2.70 GHz (the x86 build machine), "
             "the port and the reference's own single-rank build on the same inputs")
PORT_SLOWDOWN = {
    "parallel_cc": {"factor": 1.07, "reference_s": 0.359, "port_s": 0.384, "how": _PORT_HOW},
    "square_root_er1000": {"factor": 5.27, "reference_trials_per_s": 164.6, "port_trials_per_s": 31.2,
                           "how": _PORT_HOW},
    "square_root_k4000": {"factor": 2.15, "reference_trials_per_s": 0.220, "port_trials_per_s": 0.102,
                          "how": _PORT_HOW},
}
METRIC = "CC edges/s (parallel_cc, BA n=1,024,000 m=16)"
# init, sample_draws, 4 x sample_hook (slices of 1, 1, 2 and 4 eighths), 3 x compress4 (after all
# but the last slice), compress_giant_bitmap, filter, hook_survivors, finalize_count, scan_tiles,
# rank_roots, label_all
KERNELS_PER_QUERY = 2 + 4 + 3 + 1 + 2 + 4


def _max_over_ranks(x, world):
    """The largest x over the ranks (a job takes as long as its slowest replica); the process
    group's backend decides where the reduction runs (NCCL: on the GPU, gloo: on the host)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _workload():
    import graphgen
    return graphgen.barabasi_albert(N_VERTICES, ATTACH, GRAPH_SEED)


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        # raw samples (the JSON line carries their summary); CAC_CLOCKS_DIR keeps them elsewhere
        self.path = os.path.join(os.environ.get("CAC_CLOCKS_DIR", tempfile.gettempdir()), "clocks_bench_%d.csv" % device)

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.2)
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9 and parts[1].isdigit():
                    rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [int(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(int(r[2]) for r in rows), "reasons": reasons,
                "samples": len(rows)}


def _host_cores():
    return max(1, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1))


def _cpu_baseline(n, u, v, budget_s=12.0):
    """The oracle's restatement of the reference CC loop as `mpiexec -n 16` runs it: 16 ranks,
    their per-rank phases (slice sampling and rewrite) on one host thread each, the root's
    gather, shuffle and prefix union-find sequential; repeated for ~budget_s."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    threads = min(_host_cores(), VIRTUAL_RANKS)
    times = []
    t_end = time.perf_counter() + budget_s
    while True:
        t0 = time.perf_counter()
        count, _, rounds = pyoracle.cc_iss(n, u, v, GRAPH_SEED, VIRTUAL_RANKS, threads)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() > t_end or len(times) >= 50:
            break
    med = statistics.median(times)
    return {"value": len(u) / med, "unit": "edges/s", "cores": threads, "kind": "port",
            "sample": "the full BA-1M graph, %d runs of the oracle's restatement of "
                      "UnweightedIteratedSparseSampling::connectedComponents on %d virtual ranks, one host "
                      "thread each (%d rounds); median %.3f s" % (len(times), VIRTUAL_RANKS, rounds, med),
            "components": count, "virtual_ranks": VIRTUAL_RANKS,
            "port_vs_reference": PORT_SLOWDOWN["parallel_cc"],
            "reference_estimate": len(u) / med * PORT_SLOWDOWN["parallel_cc"]["factor"]}


def _ks_workloads():
    """The two single-graph square_root configurations: ER G(1000, 0.05) with weights in [1, 42]
    on 4 virtual ranks (mpiexec -n 4), and the complete graph K4000 with weights in [1, 42]."""
    import graphgen
    return [("square_root ER n=1000 p=0.05 w[1,42], 4 virtual ranks", graphgen.erdos_renyi(1000, 0.05, 0), 4, 5),
            ("square_root K4000 w[1,42]", graphgen.complete(4000, 0), 1, 3)]


_PORT_KEYS = {0: "square_root_er1000", 1: "square_root_k4000"}


def _ks_work_model(t, trials_per_s, entry_bytes, hbm_peak, peak_kind):
    """The Karger-Stein work model of one trial from a t-vertex root (recursion fan-out 2, children
    of max(ceil(N / sqrt 2) + 1, 128) vertices, leaves of at most 128): bytes B(t) = sum over the
    recursion nodes of [(N - N_t) 3 N + N^2 + N_t^2] entries plus N_b^2 per leaf, times the entry
    width; leaf work = sum over the leaves of N_b^3 integer operations (Stoer-Wagner). Both are
    reported against the trial rate: bytes against the measured HBM copy bandwidth, leaf work
    against the issue peak of one 32-lane instruction per SM sub-partition per cycle
    (152 SMs x 4 x 32 lanes x 2.07 GHz)."""
    entries, ops, level = 0, 0, [t]
    while level:
        nxt = []
        for nv in level:
            if nv <= 128:
                entries += nv * nv
                ops += nv ** 3
            else:
                nt = max(int(math.ceil(nv / math.sqrt(2))) + 1, 128)
                entries += (nv - nt) * 3 * nv + nv * nv + nt * nt
                nxt += [nt, nt]
        level = nxt
    b = entries * entry_bytes
    issue_peak = 152 * 4 * 32 * 2.07e9
    return {"root_vertices": t, "entry_bytes": entry_bytes, "bytes_per_trial": b,
            "achieved_gbs": b * trials_per_s / 1e9, "hbm_peak_gbs": hbm_peak, "peak": peak_kind,
            "hbm_frac": b * trials_per_s / 1e9 / hbm_peak, "leaf_ops_per_trial": ops,
            "leaf_tops": ops * trials_per_s / 1e12, "issue_peak_tops": issue_peak / 1e12,
            "issue_frac": ops * trials_per_s / issue_peak}


def _ks_also(ctx):
    """Karger-Stein trials/s of the square_root path (the other half of the metric), each next to a
    bounded sample of the oracle's CPU replay of the same trials on every host core."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    out = []
    for wi, (name, (n, u, v, w), ranks, reps) in enumerate(_ks_workloads()):
        g = ctx.graph(n, u, v, w)
        res = g.square_root(0.95, seed=0, virtual_ranks=ranks)  # warm-up (also builds the level buffers)
        ms = []
        for _ in range(reps):
            res = g.square_root(0.95, seed=0, virtual_ranks=ranks)
            ms.append(res.device_ms)
        trials = res.total_trials
        deg = np.zeros(n, np.uint64)
        np.add.at(deg, u, w.astype(np.uint64))
        np.add.at(deg, v, w.astype(np.uint64))
        # the oracle replays trials on every host core at once (trials are independent, as across
        # the reference's ranks; the C replay releases the interpreter lock)
        cores = _host_cores()
        per = res.trials_per_rank
        ids = [(r, i) for r in range(ranks) for i in range(per)]
        if n > 1000:
            ids = ids[:cores]  # K4000: one trial per core (a trial takes seconds on one core)
        t0 = time.perf_counter()
        with ThreadPoolExecutor(max_workers=cores) as pool:
            vals = list(pool.map(lambda ri: pyoracle.mincut_trial(n, u, v, w, 0, ri[0], ri[1]), ids))
        cpu_s = time.perf_counter() - t0
        cpu_cut, cpu_trials = min(vals), len(ids)
        filled = None
        if n <= 1000:
            # the same query 64 times with seeds 0..63 in one cac_mincut_batch: the GPU's trial
            # throughput once it is full (one ER(1000, 0.05) query has only 60 trials in flight)
            seeds = list(range(64))
            ctx.mincut_batch([g] * len(seeds), 0.95, seeds, ranks)  # warm-up
            t1 = time.perf_counter()
            rs = ctx.mincut_batch([g] * len(seeds), 0.95, seeds, ranks)
            bs = time.perf_counter() - t1
            filled = {"queries": len(seeds), "trials": sum(r.total_trials for r in rs),
                      "trials_per_s": sum(r.total_trials for r in rs) / bs, "ms_per_batch": bs * 1e3,
                      "timing": "host wall clock around cac_mincut_batch"}
        peak, peak_kind = _peaks()
        tps = trials / (statistics.median(ms) / 1e3)
        out.append({"workload": name, "trials": trials, "cut": int(res.cut),
                    "min_weighted_degree": int(deg.min()), "ms_per_query": statistics.median(ms),
                    "trials_per_s": tps,
                    "work_model": _ks_work_model(res.intermediate, tps, 4 if int(w.astype(np.uint64).sum()) < 2 ** 32
                                                 else 8, peak, peak_kind),
                    "cpu_baseline": {"trials_per_s": cpu_trials / cpu_s, "cores": cores, "kind": "port",
                                     "sample": "%d trial(s) of the oracle's replay on %d host threads"
                                               % (cpu_trials, cores),
                                     "cut_agrees": (cpu_cut == res.cut) if cpu_trials == trials else None,
                                     "port_vs_reference": PORT_SLOWDOWN[_PORT_KEYS[wi]],
                                     "reference_estimate_trials_per_s":
                                         cpu_trials / cpu_s * PORT_SLOWDOWN[_PORT_KEYS[wi]]["factor"]},
                    "batched_64_queries": filled})
        g.free()
    return out


def run_ks(args, rank, world):
    """--workload ks-er1000 | ks-k4000: only the square_root (Karger-Stein) measurement, one JSON line."""
    import torch
    import cac
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    name, (n, u, v, w), ranks, _ = _ks_workloads()[0 if args.workload == "ks-er1000" else 1]
    stream = torch.cuda.Stream(device=dev)
    ctx = cac.Context(dev, stream=stream.cuda_stream)
    if args.quotient_kernel:
        ctx.set_quotient_kernel(args.quotient_kernel)
    g = ctx.graph(n, u, v, w)
    for _ in range(args.warmup):
        res = g.square_root(0.95, seed=0, virtual_ranks=ranks)
    torch.cuda.synchronize()
    ms = []
    with Clocks(dev) as clk:
        for _ in range(args.steps):
            res = g.square_root(0.95, seed=0, virtual_ranks=ranks)
            ms.append(res.device_ms)
    total_ms = sum(ms)
    total_ms = _max_over_ranks(total_ms, world)
    line = {"metric": "Karger-Stein trials/s (%s)" % name, "value": world * res.total_trials * args.steps / (total_ms / 1e3),
            "unit": "trials/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u64", "data": "synthetic (seeded)", "cut": int(res.cut),
            "config": {"workload": name, "vertices": n, "edges": int(len(u)), "virtual_ranks": ranks,
                       "trials_per_query": res.total_trials, "intermediate_size": res.intermediate,
                       "quotient_kernel": args.quotient_kernel or "autotuned"},
            "clocks": clk.summary()}
    peak, peak_kind = _peaks()
    line["work_model"] = _ks_work_model(res.intermediate, res.total_trials / (total_ms / args.steps / 1e3),
                                        4 if int(w.astype(np.uint64).sum()) < 2 ** 32 else 8, peak, peak_kind)
    if rank == 0:
        print(json.dumps(line))
    g.free()
    ctx.close()
    return 0


def _ks_sparse_measure(ctx, steps, warmup):
    """Plain Karger-Stein (the karger_stein executable, p = 0.9) on a Watts-Strogatz graph with
    32,000 vertices and 512,000 edges (k = 32, rewiring 0.4, weights in [1, 100]): the shape of the
    reference's published sequential karger_stein baseline on ws_32k_16 (59.6 s median on one
    core, evaluation/data/e1/baselines.csv:2-3). The root and the upper levels are edge lists
    (sparse recursion), the levels from 2048 vertices down dense matrices. The answer is checked
    against the oracle's exact cut outside the timed region."""
    import torch
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    g = ctx.generate("watts_strogatz", seed=1, n=32000, k=32, p=0.4, wmin=1, wmax=100)
    for _ in range(warmup):
        res = g.karger_stein(0.9, seed=0)
    wall = []
    for i in range(steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = g.karger_stein(0.9, seed=i)
        wall.append(time.perf_counter() - t0)
    u, v, w = g.edges()
    exact = pyoracle.exact_mincut_noi(g.n, u, v, w)
    out = {"workload": "karger_stein, Watts-Strogatz n=32000 m=512000 (k = 32, rewiring 0.4, w in [1, 100]), p = 0.9",
           "value": res.total_trials * steps / sum(wall), "unit": "trials/s", "ms_per_query": sum(wall) / steps * 1e3,
           "steps": steps, "trials_per_query": res.total_trials, "timing": "host wall clock per query",
           "cut": int(res.cut), "exact_cut": exact, "cut_exact": int(res.cut) == exact,
           "published_reference": {"seconds_per_query": 59.6, "hardware": "Piz Daint XC50, 1 core",
                                   "source": "evaluation/data/e1/baselines.csv:2-3 (ws_32k_16, p = 0.90)"},
           "speedup_vs_published": 59.6 / (sum(wall) / steps)}
    g.free()
    return out


def run_ks_sparse(args, rank, world):
    """--workload ks-ws32k: _ks_sparse_measure as its own line."""
    import torch
    import cac
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    ctx = cac.Context(dev, stream=stream.cuda_stream)
    if args.quotient_kernel:
        ctx.set_quotient_kernel(args.quotient_kernel)
    with Clocks(dev) as clk:
        r = _ks_sparse_measure(ctx, args.steps, args.warmup)
    total_s = _max_over_ranks(r["ms_per_query"] * args.steps / 1e3, world)
    line = {"metric": "Karger-Stein trials/s (karger_stein, Watts-Strogatz n=32000 m=512000)",
            "value": world * r["trials_per_query"] * args.steps / total_s, "unit": "trials/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_s / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (device-generated Watts-Strogatz, k = 32, rewiring 0.4, w in [1, 100])",
            "config": {"workload": "karger_stein ws_32k_16 shape", "vertices": 32000, "edges": 512000,
                       "success_probability": 0.9, "trials_per_query": r["trials_per_query"],
                       "timing": "host wall clock per query"},
            "clocks": clk.summary()}
    line.update({k: r[k] for k in ("cut", "exact_cut", "cut_exact", "published_reference", "speedup_vs_published")})
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    return 0 if line["cut_exact"] else 1


def run_approx(args, rank, world):
    """--workload approx: approx_cut (success probability 0.9, 4 copies) on G(n = 10^6, M = 10^7)
    with unit weights, generated on the device; value = edges per second of the seed-replay mode
    (the reference's own draws, the command line's default on unit-weight graphs), beside the
    counter-addressed mode. CUDA events on the library stream around each query."""
    import torch
    import cac
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    ctx = cac.Context(dev, stream=stream.cuda_stream)
    g = ctx.generate("erdos_renyi_m", seed=3, n=1000000, avg_degree=20.0, wmin=1, wmax=1)
    out = {}
    with Clocks(dev) as clk:
        for mode, replay in (("seed_replay", True), ("counter", False)):
            for _ in range(args.warmup):
                g.approx_cut(0.9, seed=0, virtual_ranks=4, seed_replay=replay)
            ms = []
            for i in range(args.steps):
                res = g.approx_cut(0.9, seed=i, virtual_ranks=4, seed_replay=replay)
                ms.append(res.device_ms)
            out[mode] = {"ms_per_query": statistics.median(ms), "total_ms": sum(ms), "level": int(res.level),
                         "cut": int(res.cut)}
    total_ms = out["seed_replay"]["total_ms"]
    total_ms = _max_over_ranks(total_ms, world)
    line = {"metric": "approx_cut edges/s (G(10^6, M=10^7), unit weights, 4 virtual ranks)",
            "value": world * g.m * args.steps / (total_ms / 1e3), "unit": "edges/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded, generated on the device)",
            "config": {"workload": "approx_cut G(n=1000000, M=10000000) unit weights, p=0.9, 4 virtual ranks",
                       "vertices": g.n, "edges": g.m, "copies": int(res.copies)},
            "modes": {k: {kk: vv for kk, vv in v.items() if kk != "total_ms"} for k, v in out.items()},
            "clocks": clk.summary()}
    if rank == 0:
        print(json.dumps(line))
    g.free()
    ctx.close()
    return 0


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    n, u, v, _ = _workload()
    t0 = time.perf_counter()
    base = _cpu_baseline(n, u, v, budget_s=max(5.0, 1.0 * (args.steps + args.warmup)))
    line = {"impl": "reference", "metric": METRIC, "value": base["value"], "unit": "edges/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": len(u) / base["value"] * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded Barabasi-Albert, n=1,024,000, attach 16, permuted)",
            "config": {"workload": "parallel_cc BA n=1024000 m=16 (16,383,744 edges)", "vertices": n,
                       "edges": int(len(u)), "virtual_ranks": base["virtual_ranks"]},
            "cpu_baseline": base, "e2e": {"value": base["value"], "unit": "edges/s", "h2d_bytes_per_step": 0,
                                          "d2h_bytes_per_step": 0},
            "wall_s": time.perf_counter() - t0}
    print(json.dumps(line))
    return 0


def _cc_measure(ctx, stream, g, n, hu_np, hv_np, steps, warmup, world, flush):
    """Device-resident CC queries (CUDA events) and host-to-host queries through cac_cc_edges."""
    import torch
    m = g.m
    labels = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")

    def step():
        return g.connected_components(seed=GRAPH_SEED, virtual_ranks=VIRTUAL_RANKS, out=labels)

    want_count = None
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            flush.zero_()
            want_count = step()[0]
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    edge_ms, phases = [], []
    with torch.cuda.stream(stream):
        for i in range(steps):
            flush.zero_()
            starts[i].record(stream)
            count, _, res = step()
            ends[i].record(stream)
            edge_ms.append(res.edge_pass_ms)
            phases.append((res.sample_ms, res.edge_pass_ms, res.hook_ms, res.label_ms))
            assert count == want_count
        torch.cuda.synchronize()
    total_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    total_ms = _max_over_ranks(total_ms, world)
    hl_np = torch.empty(max(n, 1), dtype=torch.int32).pin_memory().numpy().view(np.uint32)
    for _ in range(max(1, warmup)):
        ctx.cc_edges(n, hu_np, hv_np, GRAPH_SEED, VIRTUAL_RANKS, hl_np)
    e2e_ms = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = ctx.cc_edges(n, hu_np, hv_np, GRAPH_SEED, VIRTUAL_RANKS, hl_np)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        assert r.num_components == want_count
    e2e_total = sum(e2e_ms)
    e2e_total = _max_over_ranks(e2e_total, world)
    link = _link_gbs(hu_np, hv_np)
    return {"value": world * m * steps / (total_ms / 1e3), "ms_per_step": total_ms / steps,
            "e2e": {"value": world * m * steps / (e2e_total / 1e3), "unit": "edges/s", "h2d_bytes_per_step": 8 * m,
                    "d2h_bytes_per_step": 4 * n, "ms_per_step": e2e_total / steps, "link_gbs": round(link, 1),
                    "link_floor_ms": round((8 * m + 4 * n) / link / 1e6, 4)},
            "edge_avg_ms": statistics.mean(edge_ms), "components": want_count,
            "phases_ms": dict(zip(("sampling_round", "filter", "hook_survivors", "labels"),
                                  [round(statistics.mean(p[i] for p in phases), 4) for i in range(4)]))}


def _link_gbs(hu_np, hv_np, reps=5):
    """Host-to-device bandwidth of the pinned edge arrays themselves (one copy of each, CUDA events;
    best of reps): the floor of the e2e query is its bytes over this rate."""
    import torch
    hu = torch.from_numpy(hu_np.view(np.int32))
    hv = torch.from_numpy(hv_np.view(np.int32))
    du, dv = torch.empty_like(hu, device="cuda"), torch.empty_like(hv, device="cuda")
    best = 0.0
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        du.copy_(hu, non_blocking=True)
        dv.copy_(hv, non_blocking=True)
        b.record()
        b.synchronize()
        best = max(best, (hu.numel() + hv.numel()) * 4 / (a.elapsed_time(b) * 1e6))
    return best


def _pinned_u32(a):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint32).view(np.int32)).pin_memory()
    return t, t.numpy().view(np.uint32)


def _rmat22(ctx, stream, steps, warmup, world, flush):
    """CC edges/s on R-MAT scale 22 (edge factor 16, a=0.57 b=0.19 c=0.19, isolated vertices kept),
    generated on the device."""
    t0 = time.perf_counter()
    g = ctx.generate("rmat", seed=GRAPH_SEED, scale=22, edge_factor=16)
    gen_s = time.perf_counter() - t0
    u, v, _ = g.edges()
    keep = (_pinned_u32(u), _pinned_u32(v))
    r = _cc_measure(ctx, stream, g, g.n, keep[0][1], keep[1][1], steps, warmup, world, flush)
    r.update({"workload": "parallel_cc R-MAT scale 22 (4,194,304 vertices, 67,108,864 edges)", "unit": "edges/s",
              "vertices": g.n, "edges": g.m, "generate_s": round(gen_s, 3)})
    g.free()
    return r


def run_cac(args, rank, world):
    import torch
    import cac

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    ctx = cac.Context(dev, stream=stream.cuda_stream)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    if args.workload == "cc-rmat22":
        with Clocks(dev) as clk:
            r = _rmat22(ctx, stream, args.steps, args.warmup, world, flush)
        line = {"metric": "CC edges/s (parallel_cc, R-MAT scale 22)", "value": r["value"], "unit": "edges/s",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
                "data": "synthetic (R-MAT generated on the device, seed 0)",
                "config": {"workload": r["workload"], "vertices": r["vertices"], "edges": r["edges"],
                           "virtual_ranks": VIRTUAL_RANKS, "l2": "flushed (512 MB write) before every timed query"},
                "e2e": r["e2e"], "components": r["components"], "phases_ms": r["phases_ms"],
                "gpu_launches": KERNELS_PER_QUERY * args.steps, "clocks": clk.summary()}
        if rank == 0:
            print(json.dumps(line))
        ctx.close()
        return 0

    n, u, v, _ = _workload()
    m = len(u)
    g = ctx.graph(n, u, v)
    hu, hu_np = _pinned_u32(u)
    hv, hv_np = _pinned_u32(v)
    with Clocks(dev) as clk:
        r = _cc_measure(ctx, stream, g, n, hu_np, hv_np, args.steps, args.warmup, world, flush)
    peak, peak_kind = _peaks()
    # whole query: 8 m bytes of edges read once + 8 n (parent initialised, label written)
    query_bytes = 8 * m + 8 * n
    query_gbs = query_bytes / (r["ms_per_step"] / 1e3) / 1e9
    filt_bytes = 8 * m
    filt_gbs = filt_bytes / (r["edge_avg_ms"] / 1e3) / 1e9
    traffic = {}
    for key, name in (("query", "cc_query_ba1m.json"), ("filter", "cc_filter_ba1m.json")):
        prof = os.path.join(ROOT, "profiles", name)
        if os.path.exists(prof):
            with open(prof) as f:
                traffic[key] = json.load(f).get("dram_bytes_per_launch")
    if rank != 0:
        g.free()
        ctx.close()
        return 0
    line = {
        "metric": METRIC, "value": r["value"], "unit": "edges/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded Barabasi-Albert, n=1,024,000, attach 16, "
                                                     "permuted)",
        "config": {"workload": "parallel_cc BA n=1024000 m=16 (16,383,744 edges)", "vertices": n, "edges": m,
                   "virtual_ranks": VIRTUAL_RANKS, "l2": "flushed (512 MB write) before every timed query",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": r["e2e"],
        "roofline": {"bound": "hbm", "scope": "whole query (%d kernels)" % KERNELS_PER_QUERY,
                     "achieved": query_gbs, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": query_gbs / peak, "traffic": traffic.get("query"), "alg_bytes_per_launch": query_bytes,
                     "avg_launch_ms": r["ms_per_step"],
                     "filter_kernel": {"kernel": "cc_filter", "achieved": filt_gbs, "frac": filt_gbs / peak,
                                       "traffic": traffic.get("filter"), "alg_bytes_per_launch": filt_bytes,
                                       "avg_launch_ms": r["edge_avg_ms"]}},
        "gpu_launches": KERNELS_PER_QUERY * args.steps,
        "phases_ms": r["phases_ms"],
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = _cpu_baseline(n, u, v)
    if not args.no_rmat:
        rr = _rmat22(ctx, stream, max(3, args.steps // 4), 3, 1, flush)
        line["also_cc_rmat22"] = {k: rr[k] for k in ("workload", "value", "unit", "ms_per_step", "e2e", "components",
                                                     "phases_ms", "generate_s")}
    if not args.no_ks:
        line["also_ks"] = _ks_also(ctx)
        line["also_ks_sparse"] = _ks_sparse_measure(ctx, 2, 1)
    g.free()
    if not args.no_batch:
        line["also_batch"] = _batch_measure(ctx, 512, 2, 1, check_exact=True)
    ctx.close()
    if not args.no_serve:
        line["also_serve"] = _serve_measure(dev, 100, (0.6,))
        # small queries only (10^3 - 10^5 edges): launch and synchronisation costs dominate the
        # plain path, so folding concurrent queries into shared launches has the most to gain
        line["also_serve_small"] = _serve_measure(dev, 300, (0.6,), m_hi=1e5)
    print(json.dumps(line))
    return 0


SERVE_NOTE = ("served graphs have n = floor(2 sqrt(m)), so square_root's pre-contraction target "
              "ceil(2 sqrt(m) + 1) is at least n and a query is the Karger-Stein budget on the whole graph (a "
              "handful of trials); sparse shapes with 10^5 - 10^6 trials per query are not in the served mix")


def _batch_measure(ctx, count, steps, warmup, check_exact=False):
    """square_root on the first `count` graphs of the uneven population in one cac_mincut_batch
    (host wall clock per batch), next to the plain path (one cac_mincut call per graph) on up to
    256 of them; every batched cut equals the plain one, and with check_exact also the exact
    minimum cut (the oracle's exact routine on every host thread, outside the timed region)."""
    import torch
    import workloads
    specs = workloads.uneven_population(4096)[:count]
    t0 = time.perf_counter()
    graphs = [workloads.make(ctx, sp) for sp in specs]
    gen_s = time.perf_counter() - t0
    seeds = [sp["seed"] for sp in specs]
    sub = min(len(graphs), 256)
    ctx.mincut_batch(graphs[:16], 0.9, seeds=seeds[:16])  # warm-up of both paths
    for g, sd in zip(graphs[:4], seeds[:4]):
        g.square_root(0.9, seed=sd)
    t0 = time.perf_counter()
    plain = [g.square_root(0.9, seed=sd) for g, sd in zip(graphs[:sub], seeds[:sub])]
    plain_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    bsub = ctx.mincut_batch(graphs[:sub], 0.9, seeds=seeds[:sub])
    bsub_s = time.perf_counter() - t0
    equal = all(a.cut == b.cut and a.total_trials == b.total_trials for a, b in zip(plain, bsub))
    for _ in range(warmup):
        res = ctx.mincut_batch(graphs, 0.9, seeds=seeds)
    wall = []
    for _ in range(steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = ctx.mincut_batch(graphs, 0.9, seeds=seeds)
        wall.append(time.perf_counter() - t0)
    exact = None
    if check_exact:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle
        want = pyoracle.exact_mincut_many([workloads.host_arrays(sp) for sp in specs], threads=_host_cores())
        exact = sum(int(r.cut) == x for r, x in zip(res, want))
    trials = sum(r.total_trials for r in res)
    total_s = sum(wall)
    out = {"workload": "uneven square_root batch (Watts-Strogatz and G(n, M), n log-uniform in [64, 8192], "
                       "w in [1, 100], p = 0.9)",
           "graphs": len(graphs), "edges": int(sum(g.m for g in graphs)), "trials_per_batch": trials,
           "value": trials * steps / total_s, "unit": "trials/s", "ms_per_step": total_s / steps * 1e3,
           "steps": steps, "queries_per_s": len(graphs) * steps / total_s,
           "device_ms_per_batch": float(res[0].device_ms), "timing": "host wall clock per batch",
           "plain_path_subset": {"graphs": sub, "trials": sum(r.total_trials for r in plain),
                                 "one_call_per_graph_s": plain_s, "batched_s": bsub_s,
                                 "plain_queries_per_s": sub / plain_s, "batched_queries_per_s": sub / bsub_s,
                                 "speedup": plain_s / bsub_s},
           "results_equal_plain": equal,
           "cuts_exact": None if exact is None else "%d of %d" % (exact, len(graphs)),
           "generate_s": round(gen_s, 3)}
    for g in graphs:
        g.free()
    return out


def run_batch(args, rank, world):
    """--workload ks-batch: square_root on a population of uneven graphs (4096 by default) in one
    batch, next to the plain path (one cac_mincut call per graph) on a subset of the same graphs."""
    import torch
    import cac
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    ctx = cac.Context(dev, stream=stream.cuda_stream)
    if args.quotient_kernel:
        ctx.set_quotient_kernel(args.quotient_kernel)
    with Clocks(dev) as clk:
        r = _batch_measure(ctx, args.graphs, args.steps, args.warmup, check_exact=args.check_exact)
    total_s = r["ms_per_step"] * args.steps / 1e3
    total_s = _max_over_ranks(total_s, world)
    line = {"metric": "Karger-Stein trials/s (square_root, %d uneven graphs in one batch)" % r["graphs"],
            "value": world * r["trials_per_batch"] * args.steps / total_s, "unit": "trials/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_s / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (device-generated Watts-Strogatz and G(n, M), seeds base + index)",
            "config": {"workload": "uneven square_root batch", "graphs": r["graphs"], "edges": r["edges"],
                       "trials_per_batch": r["trials_per_batch"], "success_probability": 0.9,
                       "n_range": [64, 8192], "timing": "host wall clock per batch",
                       "quotient_kernel": args.quotient_kernel or "autotuned"},
            "queries_per_s": world * r["graphs"] * args.steps / total_s,
            "device_ms_per_batch": r["device_ms_per_batch"], "plain_path_subset": r["plain_path_subset"],
            "results_equal_plain": r["results_equal_plain"], "cuts_exact": r["cuts_exact"],
            "generate_s": r["generate_s"], "clocks": clk.summary()}
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    return 0 if r["results_equal_plain"] else 1


def _percentile(xs, q):
    xs = sorted(xs)
    if not xs:
        return None
    k = min(len(xs) - 1, max(0, int(math.ceil(q / 100.0 * len(xs))) - 1))
    return xs[k]


def _serve_measure(dev, queries, fracs, m_hi=1e7):
    """A mixed stream of square_root : approx_cut : parallel_cc = 2:1:1 queries over 32 graphs of
    10^3 - 10^7 edges, served by cac_server under a 120 GB HBM budget: queries/s at saturation
    (every query submitted at once), the plain path (one single-query call after another) on the
    same trace, and p50/p99 latency and per-query slowdown (latency / time alone) when the same
    queries arrive as a Poisson stream at each fraction of the saturated rate."""
    import threading
    import cac
    import workloads
    specs = workloads.served_population(32, m_hi=m_hi)
    ctx = cac.Context(dev)
    srv = cac.Server(dev, hbm_budget_bytes=120 << 30)
    cg = [workloads.make(ctx, sp) for sp in specs]
    sg = []
    for sp in specs:
        d = dict(sp)
        sg.append(srv.generate(d.pop("family"), **d))
    probs = {"square_root": 0.95, "approx_cut": 0.9, "parallel_cc": 0.0}

    def plain_one(kind, gi, sd):
        g = cg[gi]
        if kind == "square_root":
            r = g.square_root(probs[kind], seed=sd)
            return (int(r.cut), int(r.trials_per_rank))
        if kind == "approx_cut":
            r = g.approx_cut(probs[kind], seed=sd)
            return (int(r.cut), int(r.trials))
        return (int(g.connected_components(seed=sd, labels=False)[0]),)

    def served_value(kind, resp):
        if kind == "parallel_cc":
            return (int(resp.num_components),)
        return (int(resp.cut), int(resp.trials))

    trace = workloads.served_trace(queries, len(specs), None, seed=7)
    for kind in ("square_root", "approx_cut", "parallel_cc"):  # warm-up
        plain_one(kind, 0, 1)
        srv.poll(srv.submit(kind, sg[0], probs[kind], 1))
    t0 = time.perf_counter()
    plain_lat, want = [], []
    for _, kind, gi, sd in trace:
        q0 = time.perf_counter()
        want.append(plain_one(kind, gi, sd))
        plain_lat.append((time.perf_counter() - q0) * 1e3)
    plain_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    tickets = [srv.submit(kind, sg[gi], probs[kind], sd) for _, kind, gi, sd in trace]
    got = [srv.poll(t)[0] for t in tickets]
    sat_s = time.perf_counter() - t0
    sat_lat = [r.queue_ms + r.service_ms for r in got]
    equal = all(served_value(kind, r) == w for (_, kind, _, _), r, w in zip(trace, got, want))
    gaps = workloads.served_trace(queries, len(specs), 1.0, seed=8)

    def poisson(frac):
        rate = frac * len(trace) / sat_s
        at = [g[0] / rate for g in gaps]
        tickets = [None] * len(trace)

        def submitter():
            start = time.perf_counter()
            for i, (_, kind, gi, sd) in enumerate(trace):
                delay = start + at[i] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                tickets[i] = srv.submit(kind, sg[gi], probs[kind], sd)

        t0 = time.perf_counter()
        th = threading.Thread(target=submitter)
        th.start()
        th.join()
        res = [srv.poll(t)[0] for t in tickets]
        span = time.perf_counter() - t0
        lat = [r.queue_ms + r.service_ms for r in res]
        slow = [x / max(p, 1e-3) for x, p in zip(lat, plain_lat)]
        by_kind = {}
        for (_, kind, _, _), x in zip(trace, lat):
            by_kind.setdefault(kind, []).append(x)
        worst = sorted(range(len(trace)), key=lambda i: -lat[i])[:5]
        ok = all(served_value(kind, r) == w for (_, kind, _, _), r, w in zip(trace, res, want))
        return ok, {"rate_per_s": rate, "queries_per_s": len(trace) / span, "p50_ms": _percentile(lat, 50),
                    "p99_ms": _percentile(lat, 99),
                    "p99_ms_by_kind": {k: _percentile(v, 99) for k, v in by_kind.items()},
                    "slowdown_p50": _percentile(slow, 50), "slowdown_p99": _percentile(slow, 99),
                    "slowest": [{"kind": trace[i][1], "edges": int(cg[trace[i][2]].m),
                                 "alone_ms": round(plain_lat[i], 3), "queue_ms": round(res[i].queue_ms, 3),
                                 "service_ms": round(res[i].service_ms, 3)} for i in worst]}

    out = {"workload": "served mixed stream (square_root : approx_cut : parallel_cc = 2:1:1, 10^3-%.0e edges, "
                       "G(n, p) and R-MAT, w in [1, 42], 120 GB budget)" % m_hi,
           "graphs": len(specs), "queries": len(trace),
           "edges_range": [int(min(g.m for g in cg)), int(max(g.m for g in cg))],
           "value": len(trace) / sat_s, "unit": "queries/s",
           "saturation": {"queries_per_s": len(trace) / sat_s, "p50_ms": _percentile(sat_lat, 50),
                          "p99_ms": _percentile(sat_lat, 99)},
           "plain_path": {"queries_per_s": len(trace) / plain_s, "p50_ms": _percentile(plain_lat, 50),
                          "p99_ms": _percentile(plain_lat, 99)},
           "speedup_vs_plain": plain_s / sat_s, "note": SERVE_NOTE}
    for frac in fracs:
        ok, r = poisson(frac)
        equal = equal and ok
        out["poisson_%dpct" % round(frac * 100)] = r
    out["results_equal_plain"] = equal
    srv.close()
    ctx.close()
    return out


def run_serve(args, rank, world):
    """--workload serve: the served mixed stream (see _serve_measure) at saturation and as Poisson
    streams at 30% and 60% of the saturated rate."""
    import torch
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    with Clocks(dev) as clk:
        r = _serve_measure(dev, args.queries, (0.3, 0.6))
    line = {"metric": "served queries/s (square_root : approx_cut : parallel_cc = 2:1:1, 10^3-10^7 edges)",
            "value": r["value"], "unit": "queries/s", "n_gpus": 1, "steps": r["queries"], "warmup": 3,
            "ms_per_step": 1e3 / r["value"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic (device-generated G(n, p) and R-MAT)",
            "config": {"workload": "served mixed stream", "graphs": r["graphs"], "edges_range": r["edges_range"],
                       "hbm_budget_bytes": 120 << 30, "queries": r["queries"]},
            "clocks": clk.summary()}
    line.update({k: r[k] for k in ("saturation", "poisson_30pct", "poisson_60pct", "plain_path", "speedup_vs_plain",
                                   "results_equal_plain", "note")})
    if rank == 0:
        print(json.dumps(line))
    return 0 if r["results_equal_plain"] else 1


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="default 20 (cc), 10 (ks-er1000, ks-k4000), 3 (ks-batch)")
    ap.add_argument("--warmup", type=int, default=None, help="default 5 (cc), 3 otherwise")
    ap.add_argument("--impl", default="cac", choices=["cac", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ks", action="store_true", help="skip the square_root (Karger-Stein) measurements")
    ap.add_argument("--no-rmat", action="store_true", help="skip the R-MAT scale 22 CC measurement")
    ap.add_argument("--workload", default="cc",
                    choices=["cc", "cc-rmat22", "ks-er1000", "ks-k4000", "ks-ws32k", "ks-batch", "serve", "approx"],
                    help="cc: the benchmark line; the others: one workload's line")
    ap.add_argument("--graphs", type=int, default=4096, help="ks-batch: graphs in the batch")
    ap.add_argument("--queries", type=int, default=200, help="serve: queries in the trace")
    ap.add_argument("--check-exact", action="store_true", help="ks-batch: check every cut against the exact cut")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched min-cut measurement")
    ap.add_argument("--no-serve", action="store_true", help="skip the served-stream measurement")
    ap.add_argument("--quotient-kernel", type=int, default=0, choices=[0, 1, 2, 3, 4],
                    help="ks-er1000 / ks-k4000 / ks-batch / ks-ws32k: 0 autotuned; 1 warp per row, 2 eight warps per row, "
                         "3 warp per row with bulk-copy staging forced for every Karger-Stein step; 4 the fixed "
                         "size rule without timing (a profiling aid: under ncu the autotuner's timings are distorted)")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = {"cc": 20, "cc-rmat22": 20, "ks-batch": 3, "ks-ws32k": 3}.get(args.workload, 10)
    if args.warmup is None:
        args.warmup = 5 if args.workload == "cc" else 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if world > 1:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        torch.distributed.init_process_group("nccl")
    try:
        if args.workload in ("ks-er1000", "ks-k4000"):
            return run_ks(args, rank, world)
        if args.workload == "ks-batch":
            return run_batch(args, rank, world)
        if args.workload == "ks-ws32k":
            return run_ks_sparse(args, rank, world)
        if args.workload == "serve":
            return run_serve(args, rank, world)
        if args.workload == "approx":
            return run_approx(args, rank, world)
        return run_cac(args, rank, world)
    finally:
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
