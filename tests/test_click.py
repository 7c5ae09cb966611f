"""CLICK, the reference's in-memory test graph (src/input/CLICK.hpp:10-49 on every rank, as
approx_cut loads it): the library's host generator against the graphs that the reference's own
generator made (tests/golden/click.json, from oracle/refbuild's click_edges harness). Host code
only: no device is needed."""
import numpy as np
import pytest

from conftest import digest


def test_click_graphs_equal_the_reference(golden, libcac):
    for case in golden("click.json"):
        n, u, v, w = libcac.click_edges(case["n"], case["ranks"], case["seed"])
        assert n == case["n"] and len(u) == case["m"], case
        assert int(w.astype(np.uint64).sum()) == case["total_weight"]
        assert [[int(a), int(b), int(c)] for a, b, c in zip(u[:4], v[:4], w[:4])] == case["first"]
        assert digest(np.concatenate([u, v, w])) == case["edges_sha256"], case


def test_click_leftover_edges_belong_to_no_rank(libcac):
    # 101 vertices: 5050 enumerated pairs over 3 ranks; the 5050 mod 3 = 1 leftover is not generated
    _, u, _, _ = libcac.click_edges(101, 3, 7)
    assert len(u) == 5049
    _, u1, _, _ = libcac.click_edges(101, 1, 7)
    assert len(u1) == 5050


def test_click_rejects_bad_sizes(libcac):
    with pytest.raises(libcac.CacError):
        libcac.click_edges(1)
    with pytest.raises(libcac.CacError):
        libcac.click_edges(100000)  # more than 2^32 - 1 pairs
