"""The drop-in command lines keep the reference's argument rules and CSV lines
(src/executables/square_root.cpp:7-40, parallel_cc.cpp:8-60, approx_cut.cpp:7-38,
karger_stein.cpp:9-47, seq_square_root.cpp:5-34)."""
import os
import subprocess

import numpy as np
import pytest

import graphgen
import pyoracle as O
from conftest import PKG, make_graph

BIN = os.path.join(PKG, "bin")


def _run(name, *args, env=None):
    e = dict(os.environ)
    for k, val in (env or {}).items():  # None: the variable is unset
        if val is None:
            e.pop(k, None)
        else:
            e[k] = val
    return subprocess.run([os.path.join(BIN, name)] + [str(a) for a in args], capture_output=True, text=True,
                          env=e, timeout=600)


@pytest.fixture(scope="module", autouse=True)
def _built(libcac):
    for name in ("square_root", "parallel_cc", "approx_cut", "karger_stein", "seq_square_root"):
        assert os.path.exists(os.path.join(BIN, name)), "command lines not built"


@pytest.mark.parametrize("name,args,usage", [
    ("square_root", ["0.95"], "Usage: square_root PROBABILITY INPUT_FILE|CLICK [SIZE] SEED"),
    ("parallel_cc", ["x"], "Usage: connected_components INPUT_FILE SEED [ITERATONS]"),
    ("approx_cut", ["0.9", "x"], "Usage: slimGraph-Light PROBABILITY INPUT_FILE|CLICK [SIZE] SEED"),
    ("karger_stein", ["x"], "Usage: karger_stein INPUT_FILE SEED"),
    ("seq_square_root", ["0.9", "x"], "Usage: square_root PROBABILITY INPUT_FILE SEED"),
])
def test_usage_on_wrong_argument_count(name, args, usage):
    r = _run(name, *args)
    assert r.returncode == 1
    assert r.stdout.strip() == usage


def _write(tmp_path, name, n, u, v, w):
    p = str(tmp_path / name)
    graphgen.write_graph(p, n, np.asarray(u, np.uint32), np.asarray(v, np.uint32), np.asarray(w, np.uint32), name)
    return p


@pytest.mark.gpu
def test_square_root_csv(golden, tmp_path):
    for name, r in golden("ref_test_inputs.json").items():
        if name.startswith("cc_"):
            continue
        path = _write(tmp_path, name, r["n"], r["u"], r["v"], r["w"])
        out = _run("square_root", "0.95", path, "0", env={"CAC_VIRTUAL_RANKS": "4"})
        assert out.returncode == 0, out.stderr
        f = out.stdout.strip().split(",")
        assert len(f) == 10 and f[0] == path and f[1] == "0" and f[2] == "4"
        assert int(f[3]) == r["n"] and int(f[4]) == len(r["u"])
        assert f[8] in ("low", "high")
        assert int(f[9]) == r["exact_cut"]
        assert int(f[7]) == -(-O.number_of_trials(r["n"], len(r["u"]), 0.95) // 4)


@pytest.mark.gpu
def test_parallel_cc_csv_iterations(golden, tmp_path):
    r = golden("ref_test_inputs.json")["cc_13.graph"]
    path = _write(tmp_path, "cc_13.graph", r["n"], r["u"], r["v"], r["w"])
    out = _run("parallel_cc", path, "7", "3")
    assert out.returncode == 0, out.stderr
    lines = out.stdout.strip().splitlines()
    assert len(lines) == 3
    for i, line in enumerate(lines):
        f = line.split(",")
        assert f[0] == path and int(f[1]) == 7 + i and f[2] == "1" and f[7] == "cc" and int(f[8]) == 5


@pytest.mark.gpu
def test_approx_cut_csv(golden, tmp_path):
    r = golden("ref_test_inputs.json")["complete_4.graph"]
    path = _write(tmp_path, "k4.graph", r["n"], r["u"], r["v"], r["w"])
    out = _run("approx_cut", "0.9", path, "3")
    assert out.returncode == 0, out.stderr
    f = out.stdout.strip().split(",")
    want, level = O.approx_cut(r["n"], r["u"], r["v"], r["w"], 0.9, 3, 1)
    assert len(f) == 9 and int(f[8]) == want and int(f[7]) == 4 * level


@pytest.mark.gpu
def test_approx_cut_seed_replay_prints_the_reference_line(golden, tmp_path):
    """CAC_SEED_REPLAY=1: the answer the reference's approx_cut printed for the same file and seed."""
    import numpy as np
    spec = next(r for r in golden("approx_stream.json")["runs"] if r["name"] == "er_400")
    n, u, v, _ = make_graph(spec)
    path = _write(tmp_path, "er400.in", n, u, v, np.ones_like(u))
    for sd in (0, 5, 11):
        for mode in ("1", None):  # required, and the default on a unit-weight graph
            out = _run("approx_cut", "0.9", path, sd, env={"CAC_SEED_REPLAY": mode})
            assert out.returncode == 0, out.stderr
            f = out.stdout.strip().split(",")
            assert int(f[8]) == spec["weights"][sd]
            assert int(f[7]) == 4 * (spec["weights"][sd].bit_length() - 1)
        # turned off: the counter-addressed keep test
        out = _run("approx_cut", "0.9", path, sd, env={"CAC_SEED_REPLAY": "0"})
        want, level = O.approx_cut(n, u, v, np.ones_like(u), 0.9, sd, 1)
        f = out.stdout.strip().split(",")
        assert out.returncode == 0 and int(f[8]) == want and int(f[7]) == 4 * level
    # a weighted graph: the counter-addressed test by default, a clean failure when the replay is required
    r = golden("ref_test_inputs.json")["complete_4.graph"]
    wpath = _write(tmp_path, "k4.graph", r["n"], r["u"], r["v"], r["w"])
    out = _run("approx_cut", "0.9", wpath, "3", env={"CAC_SEED_REPLAY": "1"})
    assert out.returncode == 1 and "weight" in out.stderr


@pytest.mark.gpu
def test_malformed_file_fails_cleanly(tmp_path):
    p = tmp_path / "bad.graph"
    p.write_text("hdr\n5 2\n0 1 1\n")
    out = _run("square_root", "0.95", str(p), "0")
    assert out.returncode == 1 and "malformed" in out.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("ranks", ["1", "3"])
def test_click_square_root_and_approx_cut(golden, ranks):
    # the in-memory CLICK graph: the CSV line reports n and the n (n - 1) / 2 enumerated pairs, and
    # square_root's answer is the exact minimum cut of the graph the reference generates
    case = next(c for c in golden("click.json") if c["n"] == 101 and c["ranks"] == 3)
    seed = str(case["seed"])
    out = _run("square_root", "0.95", "CLICK", "101", seed, env={"CAC_VIRTUAL_RANKS": ranks})
    f = out.stdout.strip().split(",")
    assert out.returncode == 0, out.stderr
    assert f[0] == "CLICK" and f[1] == seed and f[2] == ranks and f[3] == "101" and f[4] == "5050"
    if ranks == "3":
        assert int(f[-1]) == case["exact_cut"]
    out = _run("approx_cut", "0.9", "CLICK", "101", seed, env={"CAC_VIRTUAL_RANKS": ranks})
    assert out.returncode == 0, out.stderr
    f = out.stdout.strip().split(",")
    assert f[0] == "CLICK" and f[3] == "101" and f[4] == "5050" and int(f[-1]) >= 1


@pytest.mark.gpu
def test_karger_stein_csv(golden, tmp_path):
    # input,seed,1,n,m,time,?,co-karger-stein,cut; the cut equals the reference executable's
    for name, r in golden("ref_test_inputs.json").items():
        if name.startswith("cc_"):
            continue
        path = _write(tmp_path, name, r["n"], r["u"], r["v"], r["w"])
        out = _run("karger_stein", path, "0")
        assert out.returncode == 0, out.stderr
        f = out.stdout.strip().split(",")
        assert len(f) == 9 and f[0] == path and f[1:3] == ["0", "1"] and f[6:8] == ["?", "co-karger-stein"]
        assert int(f[3]) == r["n"] and int(f[4]) == len(r["u"]) and float(f[5]) >= 0
        assert int(f[8]) == r["karger_stein_cut"]


@pytest.mark.gpu
def test_seq_square_root_csv(golden, tmp_path):
    # input,seed,1,n,m,cuttingTime,mpiTime,trials,low,weight: the one-process square_root
    spec = golden("mincut_seeded.json")[1]
    n, u, v, w = make_graph(spec)
    path = _write(tmp_path, spec["name"], n, u, v, w)
    out = _run("seq_square_root", "0.95", path, "3")
    assert out.returncode == 0, out.stderr
    f = out.stdout.strip().split(",")
    assert len(f) == 10 and f[0] == path and f[1:3] == ["3", "1"] and f[6] == "0.000000" and f[8] == "low"
    assert int(f[3]) == n and int(f[4]) == len(u)
    assert int(f[7]) == spec["square_root_trials"] and int(f[9]) == spec["exact_cut"]
    # the same trials and answer as square_root on one virtual rank
    one = _run("square_root", "0.95", path, "3", env={"CAC_VIRTUAL_RANKS": "1"}).stdout.strip().split(",")
    assert one[7] == f[7] and one[9] == f[9]


@pytest.mark.gpu
def test_command_lines_read_the_binary_cache(golden, tmp_path, libcac):
    # the same answers from the text file and from its cache
    spec = golden("mincut_seeded.json")[0]
    n, u, v, w = make_graph(spec)
    text = _write(tmp_path, "g.in", n, u, v, w)
    cache = str(tmp_path / "g.cacg")
    libcac.cache_convert(text, cache)
    for name, args in (("square_root", ["0.95"]), ("approx_cut", ["0.9"]), ("parallel_cc", [])):
        a = _run(name, *args, text, "1").stdout.strip().split(",")
        b = _run(name, *args, cache, "1").stdout.strip().split(",")
        assert a and b and a[3:5] == b[3:5] and a[-1] == b[-1], (name, a, b)
    assert int(_run("square_root", "0.95", cache, "0").stdout.strip().split(",")[-1]) == spec["exact_cut"]
