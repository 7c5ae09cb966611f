"""Regenerates the golden fixtures of tests/golden/ from the reference itself.

Runs the reference's own code, compiled unmodified by oracle/refbuild into oracle/_ref/
(single-rank MPI stand-in + union-by-rank disjoint-sets stand-in), on
  * the reference's known-answer inputs (test_inputs/*.graph),
  * seeded synthetic graphs from graphgen (regenerated from their specs at test time),
and records its outputs. Only runs where the reference tree is mounted; its root comes from
--reference, else $CAC_REFERENCE_ROOT, else the build container's mount point:

    make -C oracle/refbuild REF=<tree> && python tests/golden/make_golden.py --reference <tree>
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_TREE = os.environ.get("CAC_REFERENCE_ROOT", "/root/reference")
REF_BIN = os.path.join(ROOT, "oracle", "_ref")
sys.path.insert(0, os.path.join(ROOT, "comm-avoiding-cuts-cc_gb300"))
import graphgen  # noqa: E402


def run(*args):
    return subprocess.run([os.path.join(REF_BIN, args[0])] + [str(a) for a in args[1:]], capture_output=True,
                          text=True, check=True).stdout


def labels_of(path, seed=0):
    out = run("cc_labels", path, seed).split()
    count, n = int(out[0]), int(out[1])
    return count, np.array(out[2:2 + n], dtype=np.uint32)


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u4").tobytes()).hexdigest()


def make_spec(spec):
    kind = spec["kind"]
    if kind == "er":
        return graphgen.erdos_renyi(spec["n"], spec["p"], spec["seed"], wmax=spec.get("wmax", 42))
    if kind == "er_m":
        return graphgen.erdos_renyi_m(spec["n"], spec["deg"], spec["seed"], wmax=spec.get("wmax", 100))
    if kind == "ba":
        return graphgen.barabasi_albert(spec["n"], spec["attach"], spec["seed"])
    if kind == "rmat":
        return graphgen.rmat(spec["scale"], spec["ef"], spec["seed"])
    if kind == "ws":
        return graphgen.watts_strogatz(spec["n"], spec["k"], spec["p"], spec["seed"], wmax=spec.get("wmax", 100))
    if kind == "complete":
        return graphgen.complete(spec["n"], spec["seed"], wmax=spec.get("wmax", 42))
    raise ValueError(kind)


CC_SPECS = [
    {"name": "er_sparse_5k", "kind": "er", "n": 5000, "p": 0.0002, "seed": 3, "wmax": 1},
    {"name": "er_m_20k", "kind": "er_m", "n": 20000, "deg": 1.2, "seed": 4, "wmax": 1},
    {"name": "ba_20k_3", "kind": "ba", "n": 20000, "attach": 3, "seed": 5},
    {"name": "rmat_14", "kind": "rmat", "scale": 14, "ef": 4, "seed": 6},
    {"name": "rmat_16", "kind": "rmat", "scale": 16, "ef": 16, "seed": 7},
]

CUT_SPECS = [
    {"name": "er_200", "kind": "er", "n": 200, "p": 0.08, "seed": 11},
    {"name": "ws_300_6", "kind": "ws", "n": 300, "k": 6, "p": 0.4, "seed": 12},
    {"name": "er_m_500", "kind": "er_m", "n": 500, "deg": 10, "seed": 13},
    {"name": "k_150", "kind": "complete", "n": 150, "seed": 14},
    {"name": "er_1000_c1", "kind": "er", "n": 1000, "p": 0.05, "seed": 0},
]


# graphs whose approx_cut answers (one per seed) are taken from the reference's approx_cut
# executable, to pin the replay of its own draws; "unit": every weight 1
APPROX_SPECS = [
    {"name": "er_200_dense", "kind": "er", "n": 200, "p": 0.3, "seed": 31, "wmax": 1, "unit": True},
    {"name": "er_400", "kind": "er", "n": 400, "p": 0.08, "seed": 32, "wmax": 1, "unit": True},
    {"name": "k_60", "kind": "complete", "n": 60, "seed": 33, "wmax": 1, "unit": True},
    {"name": "ws_300_24", "kind": "ws", "n": 300, "k": 24, "p": 0.3, "seed": 34, "wmax": 1, "unit": True},
    {"name": "ba_800_12", "kind": "ba", "n": 800, "attach": 12, "seed": 35, "unit": True},
    {"name": "er_200_w15", "kind": "er", "n": 200, "p": 0.06, "seed": 24, "wmax": 15},
    {"name": "er_m_600_w9", "kind": "er_m", "n": 600, "deg": 6, "seed": 25, "wmax": 9},
]
APPROX_SEEDS = list(range(16))

# (seed, level, count, weights) of the binomial_distribution draws dumped by binom_stream
BINOM_CASES = [(s, lv, cnt, ws) for s in (0, 1, 42, 4294967295)
               for lv, cnt, ws in ((1, 64, (1,)), (2, 64, (1,)), (5, 40, (1,)), (1, 50, (1, 2, 7, 15, 0)),
                                   (3, 50, (3, 14, 1)), (9, 30, (15, 1)), (40, 20, (1,)))]

# (vertices, ranks, seed) of the CLICK graphs pinned against the reference's generator
CLICK_CASES = [(2, 1, 0), (12, 2, 5), (50, 1, 0), (101, 3, 7), (120, 4, 11), (700, 5, 42), (2000, 1, 3)]

# vertex counts and success probabilities at which comincut::number_of_trials is pinned
KS_TRIAL_SIZES = [2, 100, 128, 129, 150, 181, 182, 200, 500, 1000, 2830, 4000, 16384, 100000, 1000000]
KS_TRIAL_PROBABILITIES = [0.0, 0.5, 0.9, 0.95, 0.99]


def main():
    global REF_TREE
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=REF_TREE, help="the reference's source tree")
    REF_TREE = ap.parse_args().reference
    if not os.path.isdir(REF_TREE) or not os.path.exists(os.path.join(REF_BIN, "cc_labels")):
        sys.exit("needs the reference tree and oracle/_ref (make -C oracle/refbuild)")
    # 1. sitmo known answers from the reference engine
    with open(os.path.join(HERE, "sitmo_kat.txt"), "w") as f:
        f.write(run("sitmo_kat"))
    # 2. the reference's known-answer inputs
    known = {}
    tdir = os.path.join(REF_TREE, "test_inputs")
    for fn in sorted(os.listdir(tdir)):
        path = os.path.join(tdir, fn)
        n, u, v, w = graphgen.read_graph(path)
        rec = {"n": n, "u": u.tolist(), "v": v.tolist(), "w": w.tolist()}
        if fn.startswith("cc_"):
            count, lab = labels_of(path)
            rec["cc_count"] = count
            rec["cc_labels"] = lab.tolist()
            rec["parallel_cc_csv_count"] = int(run("parallel_cc", path, 0).strip().split(",")[-1])
        else:
            rec["exact_cut"] = int(run("exact_cut", path).strip())
            rec["square_root_cut"] = int(run("square_root", 0.95, path, 0).strip().split(",")[-1])
            rec["karger_stein_cut"] = int(run("karger_stein", path, 0).strip().split(",")[-1])
            rec["approx_cut_reference"] = int(run("approx_cut", 0.9, path, 0).strip().split(",")[-1])
        known[fn] = rec
    with open(os.path.join(HERE, "ref_test_inputs.json"), "w") as f:
        json.dump(known, f, indent=1)
    # 3. seeded graphs: CC labels and min cuts from the reference
    out_cc, out_cut = [], []
    with tempfile.TemporaryDirectory() as td:
        for spec in CC_SPECS:
            n, u, v, w = make_spec(spec)
            path = os.path.join(td, spec["name"] + ".in")
            graphgen.write_graph(path, n, u, v, np.ones_like(w), spec["name"])
            count, lab = labels_of(path, 1)
            rec = dict(spec, m=int(len(u)), cc_count=count, labels_sha256=digest(lab),
                       edges_sha256=digest(np.concatenate([u, v])))
            out_cc.append(rec)
        for spec in CUT_SPECS:
            n, u, v, w = make_spec(spec)
            path = os.path.join(td, spec["name"] + ".in")
            graphgen.write_graph(path, n, u, v, w, spec["name"])
            rec = dict(spec, m=int(len(u)), edges_sha256=digest(np.concatenate([u, v, w])))
            rec["exact_cut"] = int(run("exact_cut", path).strip())
            csv = run("square_root", 0.95, path, 0).strip().split(",")
            rec["square_root_cut"] = int(csv[-1])
            rec["square_root_trials"] = int(csv[7])
            rec["karger_stein_cut"] = int(run("karger_stein", path, 0).strip().split(",")[-1])
            out_cut.append(rec)
    # 4. CLICK graphs (the reference's CLICK::generateSlice on every rank, via oracle/refbuild's
    # click_edges harness) and their exact minimum cuts
    out_click = []
    with tempfile.TemporaryDirectory() as td:
        for n, p, seed in CLICK_CASES:
            toks = run("click_edges", n, p, seed).split()
            k = int(toks[1])
            a = np.array(toks[2:2 + 3 * k], dtype=np.uint64).reshape(k, 3)
            u, v, w = (a[:, i].astype(np.uint32) for i in range(3))
            rec = dict(n=n, ranks=p, seed=seed, m=k, total_weight=int(w.astype(np.uint64).sum()),
                       edges_sha256=digest(np.concatenate([u, v, w])), first=[[int(x) for x in r] for r in a[:4]])
            if n <= 120:
                path = os.path.join(td, "click.in")
                graphgen.write_graph(path, n, u, v, w, "click")
                rec["exact_cut"] = int(run("exact_cut", path).strip())
            out_click.append(rec)
    # 5. comincut::number_of_trials, the karger_stein executable's trial count (oracle/refbuild's
    # ks_trials harness around the reference's own function)
    ks = []
    for p in KS_TRIAL_PROBABILITIES:
        for line in run("ks_trials", p, *KS_TRIAL_SIZES).splitlines():
            n, _, t = line.split()
            ks.append({"n": int(n), "p": p, "trials": int(t)})
    with open(os.path.join(HERE, "ks_trials.json"), "w") as f:
        json.dump(ks, f, indent=0)
    # 6. approx_cut on the reference's own draws: binomial_distribution draws on the sitmo engine
    # (oracle/refbuild's binom_stream harness) and the approx_cut executable's answers
    binom = []
    for seed, level, cnt, ws in BINOM_CASES:
        head, tail = run("binom_stream", seed, level, cnt, *ws).split(":")
        binom.append({"seed": seed, "level": level, "count": cnt, "weights": list(ws),
                      "draws": [int(x) for x in head.split()], "next_output": int(tail)})
    runs = []
    with tempfile.TemporaryDirectory() as td:
        for spec in APPROX_SPECS:
            n, u, v, w = make_spec(spec)
            if spec.get("unit"):
                w = np.ones_like(u)
            path = os.path.join(td, spec["name"] + ".in")
            graphgen.write_graph(path, n, u, v, w, spec["name"])
            answers = [int(run("approx_cut", 0.9, path, sd).strip().split(",")[-1]) for sd in APPROX_SEEDS]
            runs.append(dict(spec, m=int(len(u)), edges_sha256=digest(np.concatenate([u, v, w])), success_probability=0.9,
                             seeds=APPROX_SEEDS, weights=answers))
    with open(os.path.join(HERE, "approx_stream.json"), "w") as f:
        json.dump({"binomial": binom, "runs": runs}, f, indent=1)
    with open(os.path.join(HERE, "click.json"), "w") as f:
        json.dump(out_click, f, indent=1)
    with open(os.path.join(HERE, "cc_seeded.json"), "w") as f:
        json.dump(out_cc, f, indent=1)
    with open(os.path.join(HERE, "mincut_seeded.json"), "w") as f:
        json.dump(out_cut, f, indent=1)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
