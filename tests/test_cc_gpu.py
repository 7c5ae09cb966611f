"""Parity of the CUDA connected-components path with the reference's labels (through the C ABI)."""
import numpy as np
import pytest

import graphgen
import pyoracle as O
from conftest import digest, make_graph

pytestmark = pytest.mark.gpu


def test_reference_test_inputs(golden, ctx):
    ref = golden("ref_test_inputs.json")
    for name in ("cc_8.graph", "cc_13.graph"):
        r = ref[name]
        g = ctx.graph(r["n"], r["u"], r["v"], r["w"])
        for ranks in (1, 2, 4):
            count, lab, res = g.connected_components(seed=0, virtual_ranks=ranks)
            assert count == r["cc_count"] == 5
            assert lab.tolist() == r["cc_labels"]


@pytest.mark.parametrize("idx", range(5))
def test_seeded_graphs_match_reference_labels(golden, ctx, idx):
    spec = golden("cc_seeded.json")[idx]
    n, u, v, w = make_graph(spec)
    g = ctx.graph(n, u, v)
    for seed, ranks in ((1, 1), (7, 3), (2, 16)):
        count, lab, res = g.connected_components(seed=seed, virtual_ranks=ranks)
        assert count == spec["cc_count"]
        assert digest(lab) == spec["labels_sha256"]


@pytest.mark.parametrize("case", ["empty", "no_edges", "self_loops", "duplicates", "path_desc", "star", "two_paths"])
def test_edge_cases(ctx, case):
    if case == "empty":
        n, u, v = 0, [], []
    elif case == "no_edges":
        n, u, v = 7, [], []
    elif case == "self_loops":
        n, u, v = 6, [0, 3, 3, 5], [0, 3, 3, 5]
    elif case == "duplicates":
        n, u, v = 9, [1, 1, 8, 1, 8, 2], [8, 8, 1, 8, 1, 3]
    elif case == "path_desc":  # a long chain given from the high end: deep union-find paths
        n = 50000
        u = np.arange(n - 1, 0, -1, dtype=np.uint32)
        v = u - 1
    elif case == "star":
        n = 100001
        u = np.zeros(n - 1, np.uint32)
        v = np.arange(1, n, dtype=np.uint32)
    else:
        n = 40001
        u = np.concatenate([np.arange(0, 20000, 2), np.arange(1, 20001, 2)]).astype(np.uint32)
        v = (u + 2).astype(np.uint32)
    u = np.asarray(u, np.uint32)
    v = np.asarray(v, np.uint32)
    want_count, want = O.cc_labels(n, u, v)
    g = ctx.graph(n, u, v)
    count, lab, _ = g.connected_components(seed=3)
    assert count == want_count
    if n:
        assert np.array_equal(lab, want)


def test_unaligned_device_edges_and_device_labels(ctx):
    torch = pytest.importorskip("torch")
    n, u, v, _ = graphgen.erdos_renyi_m(30000, 1.5, 9, wmax=1)
    want_count, want = O.cc_labels(n, u, v)
    m = len(u)
    # device edge arrays starting 4 bytes past a 16-byte boundary take the scalar path
    du = torch.zeros(m + 1, dtype=torch.int32, device="cuda")
    dv = torch.zeros(m + 1, dtype=torch.int32, device="cuda")
    du[1:] = torch.from_numpy(u.view(np.int32)).cuda()
    dv[1:] = torch.from_numpy(v.view(np.int32)).cuda()
    torch.cuda.synchronize()
    g = ctx.graph(n, du[1:], dv[1:])
    out = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    count, lab, _ = g.connected_components(seed=0, out=out)
    torch.cuda.synchronize()
    assert count == want_count
    assert np.array_equal(out.cpu().numpy().view(np.uint32), want)


def test_repeated_runs_are_identical(ctx):
    n, u, v, _ = graphgen.rmat(16, 8, 21)
    want_count, want = O.cc_labels(n, u, v)
    g = ctx.graph(n, u, v)
    for seed in range(6):
        count, lab, _ = g.connected_components(seed=seed, virtual_ranks=1 + seed)
        assert count == want_count and np.array_equal(lab, want)


def test_replayed_queries_match(ctx):
    # the second identical query is captured into a CUDA graph, later ones replay it; a different
    # query in between must not be served by the stale capture
    n1, u1, v1, _ = graphgen.rmat(15, 8, 31)
    n2, u2, v2, _ = graphgen.erdos_renyi_m(40000, 1.1, 32, wmax=1)
    g1, g2 = ctx.graph(n1, u1, v1), ctx.graph(n2, u2, v2)
    w1, w2 = O.cc_labels(n1, u1, v1), O.cc_labels(n2, u2, v2)
    for g, (wc, wl) in [(g1, w1)] * 4 + [(g2, w2)] * 3 + [(g1, w1)] * 3:
        count, lab, _ = g.connected_components(seed=4, virtual_ranks=2)
        assert count == wc and np.array_equal(lab, wl)


def test_one_call_host_entry_point(ctx):
    n, u, v, _ = graphgen.barabasi_albert(50000, 4, 2)
    want_count, want = O.cc_labels(n, u, v)
    lab = np.zeros(n, np.uint32)
    res = ctx.cc_edges(n, u, v, seed=5, virtual_ranks=2, labels=lab)
    assert res.num_components == want_count and np.array_equal(lab, want)
    # 32-edge chunks per draw: the sampled edge count rounds each rank's budget up to a chunk
    assert 0 <= res.sampled_edges - O.cc_sample_count(n, len(u)) < 32 * 2


def _pinned(a):
    torch = pytest.importorskip("torch")
    t = torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).pin_memory()
    return t, t.numpy().view(np.uint32)


@pytest.mark.parametrize("kind", ["connected_parts", "sparse_forest"])
def test_host_entry_point_streamed_piece_paths(ctx, kind):
    # above 2 Mi edges the host edge list streams: pageable arrays (pieces in one strided copy per
    # array), pinned arrays (pieces pulled by a kernel), pinned arrays 4 bytes off a 16-byte
    # boundary (strided copy again), and a call without labels. The sparse forest's sample budget
    # covers the whole list (no gaps, no filter).
    if kind == "connected_parts":
        n0, u0, v0, _ = graphgen.erdos_renyi_m(300000, 16.0, 8)
        extra = np.arange(n0, n0 + 4000, 2, dtype=np.uint32)  # 2000 two-vertex components
        n = n0 + 4000 + 77                                      # and 77 isolated vertices
        u = np.concatenate([u0, extra]).astype(np.uint32)
        v = np.concatenate([v0, extra + 1]).astype(np.uint32)
    else:
        n, u, v, _ = graphgen.erdos_renyi_m(3000000, 1.47, 9)
    assert len(u) > (2 << 20)
    want_count, want = O.cc_labels(n, u, v)
    (ta, pua), (tb, pva) = _pinned(u), _pinned(v)
    (tc, puo), (td, pvo) = _pinned(np.concatenate([[0], u])), _pinned(np.concatenate([[0], v]))
    assert pua.ctypes.data % 16 == 0 and puo[1:].ctypes.data % 16 == 4
    lab = np.zeros(n, np.uint32)
    for hu, hv in ((u, v), (pua, pva), (puo[1:], pvo[1:])):
        for _ in range(3):  # direct, captured, replayed
            lab[:] = 0
            res = ctx.cc_edges(n, hu, hv, seed=3, labels=lab)
            assert res.num_components == want_count and np.array_equal(lab, want)
    assert ctx.cc_edges(n, pua, pva, seed=3).num_components == want_count


@pytest.mark.slow
def test_one_call_host_entry_point_streams_chunks(ctx):
    # 35 M edges from host arrays: the sample pieces are hooked as they arrive, the gaps between
    # them stream through the giant-component filter; a second, disconnected copy of the graph and
    # isolated vertices check the labels of many components. Pageable arrays (pieces through the
    # copy engine), pinned arrays (pieces read by the kernels directly) and a vertex-sorted list;
    # three calls each: run directly, captured into a graph, replayed.
    n0, u0, v0, _ = graphgen.barabasi_albert(1100000, 16, 3)
    n = 2 * n0 + 1001
    u = np.concatenate([u0, u0 + n0]).astype(np.uint32)
    v = np.concatenate([v0, v0 + n0]).astype(np.uint32)
    u, v = u[:-3], v[:-3]  # a length that is not a multiple of 4 or of the chunk
    want_count, want = O.cc_labels(n, u, v)
    order = np.lexsort((v, u))
    (tu, pu), (tv, pv) = _pinned(u), _pinned(v)
    lab = np.zeros(n, np.uint32)
    for hu, hv in ((u, v), (pu, pv), (u[order], v[order])):
        for _ in range(3):  # the staging buffers are reused by the next call
            lab[:] = 0
            res = ctx.cc_edges(n, hu, hv, labels=lab)
            assert res.num_components == want_count and np.array_equal(lab, want)
            # the pieces hold the reference's sample budget, rounded up to 256-edge pieces
            assert res.rounds == 2 and 0 <= res.sampled_edges - O.cc_sample_count(n, len(u)) < 8 * 256


@pytest.mark.slow
def test_full_size_ba_1m(ctx):
    n, u, v, _ = graphgen.barabasi_albert(1024000, 16, 0)
    assert len(u) == 16383744
    want_count, want = O.cc_labels(n, u, v)
    g = ctx.graph(n, u, v)
    count, lab, res = g.connected_components(seed=0, virtual_ranks=4)
    assert count == want_count == 1
    assert np.array_equal(lab, want)
    assert res.rounds == 2


@pytest.mark.slow
def test_full_size_rmat_scale_20(ctx):
    n, u, v, _ = graphgen.rmat(20, 16, 1)
    want_count, want = O.cc_labels(n, u, v)
    g = ctx.graph(n, u, v)
    count, lab, _ = g.connected_components(seed=1)
    assert count == want_count
    assert np.array_equal(lab, want)


@pytest.mark.parametrize("m_kind", ["copied", "streamed"])
def test_host_edges_with_an_endpoint_out_of_range(ctx, libcac, m_kind):
    # cac_cc_edges takes raw host arrays: an endpoint >= n is skipped by the kernels (every
    # endpoint is checked before it indexes) and the call fails with CAC_ERR_INVALID; the ctx
    # stays usable
    if m_kind == "copied":
        n, u, v, _ = graphgen.erdos_renyi_m(20000, 8.0, 11)
    else:
        n, u, v, _ = graphgen.erdos_renyi_m(400000, 12.0, 12)
        assert len(u) > (2 << 20)
    bad = v.copy()
    bad[len(bad) // 3] = 0xFFFFFFF0
    with pytest.raises(libcac.CacError) as e:
        ctx.cc_edges(n, u, bad)
    assert e.value.status == -1 and "endpoint" in str(e.value)
    want_count, want = O.cc_labels(n, u, v)
    lab = np.zeros(n, np.uint32)
    assert ctx.cc_edges(n, u, v, labels=lab).num_components == want_count
    assert np.array_equal(lab, want)


def test_graph_with_an_endpoint_out_of_range_is_refused(ctx, libcac):
    with pytest.raises(libcac.CacError) as e:
        ctx.graph(10, np.array([0, 3], np.uint32), np.array([1, 10], np.uint32))
    assert e.value.status == -1
    assert ctx.graph(10, np.array([0, 3], np.uint32), np.array([1, 9], np.uint32)).connected_components()[0] == 8


@pytest.mark.slow
def test_full_size_rmat_scale_22(ctx):
    """R-MAT scale 22 (4,194,304 vertices, 67,108,864 edges, generated on the device): labels
    identical to the closed-form labels, device-resident and through the one-call host entry point."""
    g = ctx.generate("rmat", seed=0, scale=22, edge_factor=16)
    n = 1 << 22
    u, v, _ = g.edges()
    assert len(u) == 67108864
    want_count, want = O.cc_labels(n, u, v)
    count, lab, _ = g.connected_components(seed=0, virtual_ranks=4)
    assert count == want_count
    assert np.array_equal(lab, want)
    lab2 = np.full(n, 0xFFFFFFFF, np.uint32)
    res = ctx.cc_edges(n, u, v, seed=0, virtual_ranks=4, labels=lab2)
    assert res.num_components == want_count and np.array_equal(lab2, want)
