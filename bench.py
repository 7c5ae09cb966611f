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
  roofline   the dominant kernel (the closing pass over all edges): algorithmic bytes 8 m per
             launch (u and v, 4 bytes each) / its CUDA-event duration, against the measured HBM
             copy bandwidth.
  cpu_baseline  the oracle's restatement of the reference's CC loop on the host, single thread.

--impl reference times the reference's CPU implementation of the path (the oracle port of
UnweightedIteratedSparseSampling::connectedComponents; the reference sources themselves are not
present on the GPU host) on the same workload and prints the same JSON line.

N > 1 (torchrun): every rank runs an independent replica of the query on its own GPU ("replicas
only": the reference's CC has no exchange that a single GPU would need); value = edges of all
ranks / max time over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "comm-avoiding-cuts-cc_gb300")
sys.path.insert(0, PKG)

import numpy as np  # noqa: E402

N_VERTICES, ATTACH, GRAPH_SEED = 1024000, 16, 0
METRIC = "CC edges/s (parallel_cc, BA n=1,024,000 m=16)"
# init, sample_draws, 8 x (sample_hook + compress4), find_giant, giant_bitmap, filter, hook_survivors,
# finalize_count, scan_tiles, rank_roots, label_all
KERNELS_PER_QUERY = 2 + 8 * 2 + 8


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
        self.path = os.path.join(ROOT, "gpurun_out", "clocks_bench_%d.csv" % device)

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


def _cpu_baseline(n, u, v, budget_s=12.0):
    """The oracle's restatement of the reference CC loop, single thread, repeated for ~budget_s."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    times = []
    t_end = time.perf_counter() + budget_s
    while True:
        t0 = time.perf_counter()
        count, _, rounds = pyoracle.cc_iss(n, u, v, GRAPH_SEED, 1)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() > t_end or len(times) >= 50:
            break
    med = statistics.median(times)
    return {"value": len(u) / med, "unit": "edges/s", "cores": 1, "kind": "port",
            "sample": "the full BA-1M graph, %d runs of the oracle's restatement of "
                      "UnweightedIteratedSparseSampling::connectedComponents (one virtual rank, %d rounds); "
                      "median %.3f s" % (len(times), rounds, med), "components": count}


def _ks_workloads():
    """The two single-graph square_root configurations: ER G(1000, 0.05) with weights in [1, 42]
    on 4 virtual ranks (mpiexec -n 4), and the complete graph K4000 with weights in [1, 42]."""
    import graphgen
    return [("square_root ER n=1000 p=0.05 w[1,42], 4 virtual ranks", graphgen.erdos_renyi(1000, 0.05, 0), 4, 5),
            ("square_root K4000 w[1,42]", graphgen.complete(4000, 0), 1, 3)]


def _ks_also(ctx):
    """Karger-Stein trials/s of the square_root path (the other half of the metric), each next to a
    bounded sample of the oracle's CPU replay of the same trials (single thread)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    out = []
    for name, (n, u, v, w), ranks, reps in _ks_workloads():
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
        t0 = time.perf_counter()
        if n <= 1000:
            cpu_cut, _ = pyoracle.square_root(n, u, v, w, 0.95, 0, ranks)
            cpu_trials = trials
        else:
            cpu_cut, cpu_trials = pyoracle.mincut_trial(n, u, v, w, 0, 0, 0), 1
        cpu_s = time.perf_counter() - t0
        out.append({"workload": name, "trials": trials, "cut": int(res.cut),
                    "min_weighted_degree": int(deg.min()), "ms_per_query": statistics.median(ms),
                    "trials_per_s": trials / (statistics.median(ms) / 1e3),
                    "cpu_baseline": {"trials_per_s": cpu_trials / cpu_s, "cores": 1, "kind": "port",
                                     "sample": "%d trial(s) of the oracle's replay" % cpu_trials,
                                     "cut_agrees": (cpu_cut == res.cut) if cpu_trials == trials else None}})
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
    if world > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    line = {"metric": "Karger-Stein trials/s (%s)" % name, "value": world * res.total_trials * args.steps / (total_ms / 1e3),
            "unit": "trials/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u64", "data": "synthetic (seeded)", "cut": int(res.cut),
            "config": {"workload": name, "vertices": n, "edges": int(len(u)), "virtual_ranks": ranks,
                       "trials_per_query": res.total_trials, "intermediate_size": res.intermediate},
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
                       "edges": int(len(u)), "virtual_ranks": 1},
            "cpu_baseline": base, "e2e": {"value": base["value"], "unit": "edges/s", "h2d_bytes_per_step": 0,
                                          "d2h_bytes_per_step": 0},
            "wall_s": time.perf_counter() - t0}
    print(json.dumps(line))
    return 0


def run_cac(args, rank, world):
    import torch
    import cac

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    n, u, v, _ = _workload()
    m = len(u)
    stream = torch.cuda.Stream(device=dev)
    ctx = cac.Context(dev, stream=stream.cuda_stream)
    g = ctx.graph(n, u, v)
    labels = torch.empty(n, dtype=torch.int32, device="cuda")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    want_count = None

    def step():
        return g.connected_components(seed=GRAPH_SEED, virtual_ranks=1, out=labels)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.zero_()
            want_count = step()[0]
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    edge_ms, phases = [], []
    with Clocks(dev) as clk, torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.zero_()
            starts[i].record(stream)
            count, _, res = step()
            ends[i].record(stream)
            edge_ms.append(res.edge_pass_ms)
            phases.append((res.sample_ms, res.edge_pass_ms, res.hook_ms, res.label_ms))
            assert count == want_count
        torch.cuda.synchronize()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * m * args.steps / (total_ms / 1e3)

    # e2e: pinned host edges -> host labels through the one-call entry point
    hu = torch.from_numpy(u.view(np.int32)).pin_memory()
    hv = torch.from_numpy(v.view(np.int32)).pin_memory()
    hl = torch.empty(n, dtype=torch.int32).pin_memory()
    hu_np = hu.numpy().view(np.uint32)
    hv_np = hv.numpy().view(np.uint32)
    hl_np = hl.numpy().view(np.uint32)
    for _ in range(max(1, args.warmup)):
        ctx.cc_edges(n, hu_np, hv_np, GRAPH_SEED, 1, hl_np)
    e2e_ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = ctx.cc_edges(n, hu_np, hv_np, GRAPH_SEED, 1, hl_np)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        assert r.num_components == want_count
    e2e_total = sum(e2e_ms)
    if world > 1:
        t = torch.tensor([e2e_total], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_total = float(t.item())
    e2e_value = world * m * args.steps / (e2e_total / 1e3)

    peak, peak_kind = _peaks()
    edge_avg_ms = statistics.mean(edge_ms)
    alg_bytes = 8 * m
    achieved = alg_bytes / (edge_avg_ms / 1e3) / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", "cc_filter_ba1m.json")
    if os.path.exists(prof):
        with open(prof) as f:
            traffic = json.load(f).get("dram_bytes_per_launch")
    if rank != 0:
        g.free()
        ctx.close()
        return 0
    line = {
        "metric": METRIC, "value": value, "unit": "edges/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded Barabasi-Albert, n=1,024,000, attach 16, "
                                                     "permuted)",
        "config": {"workload": "parallel_cc BA n=1024000 m=16 (16,383,744 edges)", "vertices": n, "edges": m,
                   "virtual_ranks": 1, "l2": "flushed (512 MB write) before every timed query",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": e2e_value, "unit": "edges/s", "h2d_bytes_per_step": 8 * m, "d2h_bytes_per_step": 4 * n,
                "ms_per_step": e2e_total / args.steps},
        "roofline": {"bound": "hbm", "kernel": "cc_filter", "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "alg_bytes_per_launch": alg_bytes, "avg_launch_ms": edge_avg_ms},
        "gpu_launches": KERNELS_PER_QUERY * args.steps,
        "phases_ms": dict(zip(("sampling_round", "filter", "hook_survivors", "labels"),
                              [round(statistics.mean(p[i] for p in phases), 4) for i in range(4)])),
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = _cpu_baseline(n, u, v)
    if not args.no_ks:
        line["also_ks"] = _ks_also(ctx)
    print(json.dumps(line))
    g.free()
    ctx.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="cac", choices=["cac", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ks", action="store_true", help="skip the square_root (Karger-Stein) measurements")
    ap.add_argument("--workload", default="cc", choices=["cc", "ks-er1000", "ks-k4000"],
                    help="cc: the benchmark line; ks-*: only one square_root configuration")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if world > 1:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        torch.distributed.init_process_group("nccl")
    try:
        if args.workload != "cc":
            return run_ks(args, rank, world)
        return run_cac(args, rank, world)
    finally:
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
