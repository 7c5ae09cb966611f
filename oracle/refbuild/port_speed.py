"""How much slower the oracle's CPU port is than the reference's own build, on one core of the
same machine and the same inputs. The GPU host runs the port as the timed CPU baseline (the
reference's sources are not there); this factor, measured where both exist, says by how much
that baseline understates the reference.

    make -C oracle/refbuild REF=<reference tree> && python oracle/refbuild/port_speed.py

Cases (single rank, so one core each):
  * parallel_cc on BA n=1,024,000, attach 16 (16,383,744 edges): the reference's parallel_cc
    executable with 5 iterations (its CSV time column, parsing excluded) against
    pyoracle.cc_iss on one virtual rank (median of 5);
  * square_root trials on ER(1000, 0.05), weights in [1, 42]: the reference's square_root
    (trials / cuttingTime) against pyoracle.mincut_trial, one thread;
  * square_root trials on K4000, weights in [1, 42] (reference: 7 trials; port: 2 trials).
Prints one JSON object; its numbers are the ones the benchmark quotes next to the port.
"""
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_BIN = os.path.join(ROOT, "oracle", "_ref")
sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "comm-avoiding-cuts-cc_gb300")]
import graphgen  # noqa: E402
import pyoracle as O  # noqa: E402


def _csv_rows(out):
    return [line.split(",") for line in out.splitlines() if line.count(",") >= 4]


def cc_case(tmp):
    n, u, v, w = graphgen.barabasi_albert(1024000, 16, 0)
    path = os.path.join(tmp, "ba1m.in")
    graphgen.write_graph(path, n, u, v, w)
    out = subprocess.run([os.path.join(REF_BIN, "parallel_cc"), path, "0", "5"], capture_output=True, text=True,
                         check=True).stdout
    # input,seed,cores,vertices,edges,time,components (one line per iteration)
    ref = statistics.median(float(r[5]) for r in _csv_rows(out))
    port = []
    for _ in range(5):
        t0 = time.perf_counter()
        O.cc_iss(n, u, v, 0, 1, 1)
        port.append(time.perf_counter() - t0)
    port = statistics.median(port)
    return {"workload": "parallel_cc BA n=1024000 m=16, 1 rank", "reference_s": ref, "port_s": port,
            "port_slowdown": port / ref}


def cut_case(tmp, name, graph, port_trials):
    n, u, v, w = graph
    path = os.path.join(tmp, "".join(c for c in name if c.isalnum()) + ".in")
    graphgen.write_graph(path, n, u, v, w)
    out = subprocess.run([os.path.join(REF_BIN, "square_root"), "0.95", path, "0"], capture_output=True, text=True,
                         check=True).stdout
    # input,seed,p,n,m,cuttingTime,mpiTime,trials,variant,weight
    r = _csv_rows(out)[-1]
    ref_tps = float(r[7]) / float(r[5])
    t0 = time.perf_counter()
    for i in range(port_trials):
        O.mincut_trial(n, u, v, w, 0, 0, i)
    port_tps = port_trials / (time.perf_counter() - t0)
    return {"workload": "square_root " + name + ", 1 rank", "reference_trials_per_s": ref_tps,
            "port_trials_per_s": port_tps, "port_slowdown": ref_tps / port_tps}


def main():
    if not os.path.exists(os.path.join(REF_BIN, "parallel_cc")):
        sys.exit("needs oracle/_ref (make -C oracle/refbuild REF=<reference tree>)")
    with tempfile.TemporaryDirectory() as tmp:
        cases = [cc_case(tmp),
                 cut_case(tmp, "ER(1000,0.05) w[1,42]", graphgen.erdos_renyi(1000, 0.05, 0), 20),
                 cut_case(tmp, "K4000 w[1,42]", graphgen.complete(4000, 0), 2)]
    print(json.dumps({"cpu": _cpu_model(), "cases": cases}, indent=1))


def _cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return None


if __name__ == "__main__":
    main()
