"""The library's edge-list reader (host code, no GPU) against the reference's format rules
(src/input/GraphInputIterator.cpp:3-36): first line skipped, `n m`, then m `u v w` triples."""
import numpy as np
import pytest

import graphgen


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_reads_reference_test_inputs(golden, libcac, tmp_path):
    for name, r in golden("ref_test_inputs.json").items():
        path = str(tmp_path / name)
        graphgen.write_graph(path, r["n"], np.array(r["u"], np.uint32), np.array(r["v"], np.uint32),
                             np.array(r["w"], np.uint32), "x")
        n, u, v, w = libcac.parse_file(path)
        assert n == r["n"] and u.tolist() == r["u"] and v.tolist() == r["v"] and w.tolist() == r["w"]


def test_multithreaded_chunks_match_numpy(libcac, tmp_path):
    n, u, v, w = graphgen.erdos_renyi_m(50000, 12, 3, wmax=1000)
    path = str(tmp_path / "big.in")
    graphgen.write_graph(path, n, u, v, w, "big")
    n2, u2, v2, w2 = libcac.parse_file(path)
    assert n2 == n and np.array_equal(u2, u) and np.array_equal(v2, v) and np.array_equal(w2, w)


def test_whitespace_is_free_form(libcac, tmp_path):
    path = _write(tmp_path, "ws.in", "# header with 1 2 3 numbers\n 4   3\n0 1 5\n\n1\t2 6\r\n2 3\n7")
    n, u, v, w = libcac.parse_file(path)
    assert n == 4 and u.tolist() == [0, 1, 2] and v.tolist() == [1, 2, 3] and w.tolist() == [5, 6, 7]


@pytest.mark.parametrize("text,status", [
    ("hdr\n4 3\n0 1 1\n1 2 1\n", -3),          # fewer lines than declared
    ("hdr\n4 1\n0 x 1\n", -3),                 # junk token
    ("hdr\n4 1\n0 9 1\n", -3),                 # endpoint >= n
    ("hdr\n4 1\n0 1 99999999999\n", -3),       # weight overflows unsigned
    ("no newline at all", -3),                 # no header line
])
def test_malformed_inputs_raise(libcac, tmp_path, text, status):
    path = _write(tmp_path, "bad.in", text)
    with pytest.raises(libcac.CacError) as e:
        libcac.parse_file(path)
    assert e.value.status == status


def test_missing_file_is_io_error(libcac, tmp_path):
    with pytest.raises(libcac.CacError) as e:
        libcac.parse_file(str(tmp_path / "nope.in"))
    assert e.value.status == -7
