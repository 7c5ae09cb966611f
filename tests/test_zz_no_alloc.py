"""cac_cc_noalloc: connected components for callers that cannot allocate device memory (a plugin
whose host framework owns all device memory, a serving path that must not take cudaMalloc's
implicit synchronisation). It runs on one fixed scratch array of the library, so this test
checks, through the C ABI, that two calls in a row on different graphs each give exactly the
labels and count of the allocating entry point cac_cc (the scratch keeps the previous call's
contents, which must not leak into the next result), and that oversized inputs are refused.
Collected last on purpose: it shares nothing with the other tests and also passes alone."""
import ctypes

import numpy as np
import pytest

import graphgen
import pyoracle as O

pytestmark = pytest.mark.gpu


def _device_u32(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint32).view(np.int32)).cuda()


def _noalloc(libcac, torch, n, u, v, offset=0, want_labels=True, want_count=True):
    """One call through the C ABI. offset > 0 places the edge arrays `offset` elements into their
    device buffers, so they are not 16-byte aligned and the scalar edge pass runs."""
    du = _device_u32(torch, np.concatenate([np.zeros(offset, np.uint32), u]))[offset:]
    dv = _device_u32(torch, np.concatenate([np.zeros(offset, np.uint32), v]))[offset:]
    labels = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    count = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    st = libcac.lib().cac_cc_noalloc(n, len(u), ctypes.c_void_p(du.data_ptr()), ctypes.c_void_p(dv.data_ptr()),
                                     ctypes.c_void_p(labels.data_ptr()) if want_labels else None,
                                     ctypes.c_void_p(count.data_ptr()) if want_count else None,
                                     ctypes.c_void_p(stream.cuda_stream))
    assert st == 0, libcac.lib().cac_last_error()
    stream.synchronize()
    return int(count.item()), labels.cpu().numpy().view(np.uint32)[:n]


def test_two_calls_in_a_row_match_cac_cc(ctx, libcac):
    torch = pytest.importorskip("torch")
    graphs = [graphgen.barabasi_albert(200000, 8, 3), graphgen.rmat(16, 8, 4)]
    for n, u, v, _ in graphs:  # two calls in a row, different graphs
        count, labels = _noalloc(libcac, torch, n, u, v)
        want_count, want_labels, _ = ctx.graph(n, u, v).connected_components(seed=0)
        assert count == want_count
        assert np.array_equal(labels, want_labels)
        assert count == O.cc_labels(n, u, v)[0]


def test_refuses_more_vertices_than_the_scratch_holds(libcac):
    lib = libcac.lib()
    st = lib.cac_cc_noalloc((1 << 22) + 1, 0, None, None, None, None, None)
    assert st == -1
    assert b"4194304" in lib.cac_last_error()


def test_endpoint_out_of_range_is_reported_in_the_count(ctx, libcac):
    # an endpoint >= n: the edge is skipped (the kernels check every endpoint before indexing)
    # and the count reads 0xFFFFFFFF; the next valid call is unaffected
    torch = pytest.importorskip("torch")
    n, u, v, _ = graphgen.erdos_renyi(5000, 0.002, 6)
    bad_v = v.copy()
    bad_v[17] = n + 3
    count, _ = _noalloc(libcac, torch, n, u, bad_v)
    assert count & 0xFFFFFFFF == 0xFFFFFFFF
    count, labels = _noalloc(libcac, torch, n, u, v)
    want_count, want = O.cc_labels(n, u, v)
    assert count == want_count and np.array_equal(labels, want)


def test_unaligned_edge_arrays_and_optional_outputs(libcac):
    # edge arrays one element past a 16-byte boundary run the scalar edge pass; either output may
    # be left out, and what is asked for is still exact
    torch = pytest.importorskip("torch")
    n, u, v, _ = graphgen.erdos_renyi_m(30000, 1.1, 7, wmax=1)
    want_count, want = O.cc_labels(n, u, v)
    count, labels = _noalloc(libcac, torch, n, u, v, offset=1)
    assert count == want_count and np.array_equal(labels, want)
    count, labels = _noalloc(libcac, torch, n, u, v, offset=3, want_labels=False)
    assert count == want_count
    assert np.all(labels == 0xFFFFFFFF)  # untouched
    count, labels = _noalloc(libcac, torch, n, u, v, want_count=False)
    assert count == -1 and np.array_equal(labels, want)


def test_no_vertices(libcac):
    # n = 0: no edges gives 0 components; any edge has an endpoint >= n, so the count reads 0xFFFFFFFF
    torch = pytest.importorskip("torch")
    empty = np.zeros(0, np.uint32)
    count, _ = _noalloc(libcac, torch, 0, empty, empty)
    assert count == 0
    count, _ = _noalloc(libcac, torch, 0, np.array([0, 1], np.uint32), np.array([1, 2], np.uint32))
    assert count & 0xFFFFFFFF == 0xFFFFFFFF
