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


# ---- binary graph cache (host code, no GPU) ----

def test_cache_round_trip_equals_text(libcac, tmp_path):
    n, u, v, w = graphgen.erdos_renyi_m(30000, 10, 7, wmax=500)
    text = str(tmp_path / "g.in")
    graphgen.write_graph(text, n, u, v, w, "g")
    cache = str(tmp_path / "g.cacg")
    libcac.cache_convert(text, cache)
    assert libcac.parse_file(cache)[0] == n
    for a, b in zip(libcac.parse_file(text), libcac.parse_file(cache)):
        assert np.array_equal(np.asarray(a), np.asarray(b))
    # header, arrays, nothing else: 32 + 3 * 4 * m bytes
    assert (tmp_path / "g.cacg").stat().st_size == 32 + 12 * len(u)


def test_cache_without_weights_reads_weights_one(libcac, tmp_path):
    n, u, v, _ = graphgen.barabasi_albert(5000, 3, 1)
    cache = str(tmp_path / "ba.cacg")
    libcac.cache_write(cache, n, u, v)
    n2, u2, v2, w2 = libcac.parse_file(cache)
    assert n2 == n and np.array_equal(u2, u) and np.array_equal(v2, v) and (w2 == 1).all()


def _corrupt(path, how):
    data = bytearray(open(path, "rb").read())
    if how == "truncated":
        data = data[:-5]
    elif how == "appended":
        data += b"\0\0\0\0"
    elif how == "weight":
        data[-1] ^= 0x01  # the last weight no longer adds up to the header's total
    elif how == "endpoint":
        data[32:36] = (0xFFFFFF00).to_bytes(4, "little")  # u[0] >= n
    open(path, "wb").write(bytes(data))


@pytest.mark.parametrize("how", ["truncated", "appended", "weight", "endpoint"])
def test_corrupted_cache_is_refused(libcac, tmp_path, how):
    n, u, v, w = graphgen.erdos_renyi_m(2000, 6, 2, wmax=9)
    cache = str(tmp_path / "c.cacg")
    libcac.cache_write(cache, n, u, v, w)
    _corrupt(cache, how)
    with pytest.raises(libcac.CacError) as e:
        libcac.parse_file(cache)
    assert e.value.status == -3


def test_text_whose_first_line_starts_with_the_magic_is_text(libcac, tmp_path):
    path = _write(tmp_path, "magic.in", "CACG is just the name of this graph\n3 2\n0 1 4\n1 2 5\n")
    n, u, v, w = libcac.parse_file(path)
    assert n == 3 and u.tolist() == [0, 1] and v.tolist() == [1, 2] and w.tolist() == [4, 5]


def test_cache_write_refuses_bad_endpoints(libcac, tmp_path):
    with pytest.raises(libcac.CacError) as e:
        libcac.cache_write(str(tmp_path / "x.cacg"), 3, np.array([0, 5]), np.array([1, 2]))
    assert e.value.status == -1


def test_cache_graph_command_line(libcac, tmp_path):
    import os
    import subprocess
    from conftest import PKG
    exe = os.path.join(PKG, "bin", "cache_graph")
    r = subprocess.run([exe, "only-one-arg"], capture_output=True, text=True)
    assert r.returncode == 1 and r.stdout.strip() == "Usage: cache_graph INPUT_FILE CACHE_FILE"
    n, u, v, w = graphgen.watts_strogatz(1000, 6, 0.3, 4, wmax=42)
    text, cache = str(tmp_path / "ws.in"), str(tmp_path / "ws.cacg")
    graphgen.write_graph(text, n, u, v, w, "ws")
    r = subprocess.run([exe, text, cache], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "%s,%d,%d" % (cache, n, len(u))
    n2, u2, v2, w2 = libcac.parse_file(cache)
    assert n2 == n and np.array_equal(u2, u) and np.array_equal(w2, w)
