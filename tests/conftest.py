import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "comm-avoiding-cuts-cc_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run on the GPU host)")
    config.addinivalue_line("markers", "slow: full-size workloads")


def _ensure_oracle():
    lib = os.path.join(ROOT, "oracle", "lib", "liboracle.so")
    if not os.path.exists(lib):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)


def _ensure_libcac():
    lib = os.path.join(PKG, "lib", "libcac.so")
    if not os.path.exists(lib):
        subprocess.run([sys.executable, os.path.join(PKG, "build.py"), "--no-oracle"], check=True)


_ensure_oracle()


@pytest.fixture(scope="session")
def golden():
    def load(name):
        with open(os.path.join(GOLDEN, name)) as f:
            return json.load(f) if name.endswith(".json") else f.read()
    return load


@pytest.fixture(scope="session")
def libcac():
    _ensure_libcac()
    import cac
    return cac


@pytest.fixture(scope="session")
def ctx(libcac):
    c = libcac.Context(0)
    yield c
    c.close()


def make_graph(spec):
    import graphgen
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


def digest(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u4").tobytes()).hexdigest()
