"""Seeded synthetic graph generators for the benchmark and test workloads.

The reference generates its inputs with NetworkX, PaRMAT and Boost generators
(utils/generate.py:10-32, input_generators/rmat_driver.sh:13-16, src/executables/er_generator.cpp);
none of those travel here, so every family is restated with counter-based integer hashing
(splitmix64 of (seed, stream, index)). Only uint64 wrap-around arithmetic is used, so a given
(family, size, seed) yields the same edge list on every machine and numpy version.

Every generator returns (n, u, v, w) with u, v, w uint32 numpy arrays (w = 1 for unweighted
families). Vertex ids are in [0, n).
"""
import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)
_GOLD = np.uint64(0x9E3779B97F4A7C15)


def _mix(z):
    z = z.astype(np.uint64, copy=True)
    with np.errstate(over="ignore"):
        z ^= z >> np.uint64(30)
        z *= np.uint64(0xBF58476D1CE4E5B9)
        z ^= z >> np.uint64(27)
        z *= np.uint64(0x94D049BB133111EB)
        z ^= z >> np.uint64(31)
    return z


def hash64(seed, stream, idx):
    """splitmix64 finaliser of seed/stream/index; idx may be an array."""
    idx = np.asarray(idx, dtype=np.uint64)
    with np.errstate(over="ignore"):
        base = _mix(np.array([(seed * 0x100000001B3 + stream * 0x9E3779B1) & 0xFFFFFFFFFFFFFFFF], dtype=np.uint64))[0]
        return _mix(idx * _GOLD + base)


def _uniform_int(seed, stream, idx, lo, hi):
    """uniform integers in [lo, hi] by multiply-shift on the top 32 bits."""
    h = hash64(seed, stream, idx) >> np.uint64(32)
    span = np.uint64(hi - lo + 1)
    return (lo + ((h * span) >> np.uint64(32))).astype(np.uint32)


def _threshold(p):
    return np.uint64(min(int(p * 2.0**64), 2**64 - 1))


def weights(seed, m, wmax, wmin=1):
    """uniform integer weights in [wmin, wmax] (stream 7)."""
    return _uniform_int(seed, 7, np.arange(m, dtype=np.uint64), wmin, wmax)


def permute_edges(seed, u, v, w):
    """seeded random permutation of the edge list (stream 9)."""
    key = hash64(seed, 9, np.arange(len(u), dtype=np.uint64))
    order = np.argsort(key, kind="stable")
    return u[order], v[order], w[order]


def erdos_renyi(n, p, seed, wmax=42, wmin=1):
    """G(n, p): every pair i < j independently with probability p (stream 1)."""
    us, vs = [], []
    thr = _threshold(p)
    for i in range(n - 1):
        j = np.arange(i + 1, n, dtype=np.uint64)
        keep = hash64(seed, 1, np.uint64(i) * np.uint64(n) + j) < thr
        vs.append(j[keep].astype(np.uint32))
        us.append(np.full(int(keep.sum()), i, dtype=np.uint32))
    u = np.concatenate(us) if us else np.zeros(0, np.uint32)
    v = np.concatenate(vs) if vs else np.zeros(0, np.uint32)
    w = weights(seed, len(u), wmax, wmin) if wmax > 1 else np.ones(len(u), np.uint32)
    return n, u, v, w


def erdos_renyi_m(n, avg_degree, seed, wmax=100, wmin=1):
    """G(n, M) with M = n * avg_degree / 2 endpoint pairs drawn uniformly (stream 2);
    self-loops are re-drawn once and dropped if they persist; parallel edges are kept
    (they merge into one heavier edge, as the reference's finalize step does)."""
    m = int(n * avg_degree // 2)
    idx = np.arange(m, dtype=np.uint64)
    u = _uniform_int(seed, 2, idx, 0, n - 1)
    v = _uniform_int(seed, 3, idx, 0, n - 1)
    loop = u == v
    v[loop] = _uniform_int(seed, 4, idx[loop], 0, n - 1)
    keep = u != v
    u, v = u[keep], v[keep]
    w = weights(seed, len(u), wmax, wmin)
    return n, u, v, w


def complete(n, seed, wmax=42, wmin=1):
    """K_n with uniform integer weights."""
    iu, ju = np.triu_indices(n, 1)
    u = iu.astype(np.uint32)
    v = ju.astype(np.uint32)
    return n, u, v, weights(seed, len(u), wmax, wmin)


def barabasi_albert(n, m_attach, seed, permute=True):
    """Preferential attachment with (n - m) * m edges, the edge count of NetworkX's
    barabasi_albert_graph(n, m) used for the reference's BA inputs. Restated as the
    Batagelj-Brandes linear-time method (each new edge copies the endpoint at a uniformly
    drawn earlier slot of the endpoint list), vectorised by pointer jumping. Multi-edges can
    occur; they do not change connectivity."""
    k = m_attach
    ne = (n - k) * k
    e = np.arange(ne, dtype=np.int64)
    src = (k + e // k).astype(np.uint32)
    # endpoint-list slots: slot 2e holds edge e's new vertex, slot 2e+1 its target. The first
    # k edges (vertex k) attach to the seed vertices 0..k-1; every later edge copies the
    # value of a uniformly drawn earlier slot in [0, 2e).
    r = hash64(seed, 5, e.astype(np.uint64)) >> np.uint64(32)
    slot = ((r * (2 * e).astype(np.uint64)) >> np.uint64(32)).astype(np.int64)
    dst = np.zeros(ne, dtype=np.uint32)
    dst[:k] = np.arange(k, dtype=np.uint32) % np.uint32(k)
    cur = slot.copy()
    todo = np.nonzero(e >= k)[0]
    while todo.size:
        c = cur[todo]
        even = (c & 1) == 0
        dst[todo[even]] = src[c[even] // 2]                 # a new-vertex slot
        odd_idx = todo[~even]
        owner = (cur[odd_idx] - 1) // 2                     # a target slot: copy its edge's target
        seed_t = owner < k
        dst[odd_idx[seed_t]] = (owner[seed_t] % k).astype(np.uint32)
        rest = odd_idx[~seed_t]
        cur[rest] = slot[owner[~seed_t]]
        todo = rest
    u = src
    v = dst
    w = np.ones(ne, dtype=np.uint32)
    if permute:
        u, v, w = permute_edges(seed, u, v, w)
    return n, u, v, w


def rmat(scale, edge_factor, seed, a=0.57, b=0.19, c=0.19, chunk=1 << 22, wmax=1, wmin=1):
    """R-MAT (Chakrabarti et al.): each of edge_factor * 2^scale edges picks one quadrant per
    bit level with probabilities a, b, c, d = 1 - a - b - c (stream 100 + level). Isolated
    vertices are kept, so n = 2^scale exactly. Unweighted unless wmax > 1."""
    n = 1 << scale
    m = edge_factor * n
    ta, tb, tc = _threshold(a), _threshold(a + b), _threshold(a + b + c)
    u = np.zeros(m, dtype=np.uint32)
    v = np.zeros(m, dtype=np.uint32)
    for s in range(0, m, chunk):
        idx = np.arange(s, min(m, s + chunk), dtype=np.uint64)
        uu = np.zeros(len(idx), dtype=np.uint32)
        vv = np.zeros(len(idx), dtype=np.uint32)
        for lvl in range(scale):
            h = hash64(seed, 100 + lvl, idx)
            bit_u = (h >= tb).astype(np.uint32)
            bit_v = (((h >= ta) & (h < tb)) | (h >= tc)).astype(np.uint32)
            uu = (uu << np.uint32(1)) | bit_u
            vv = (vv << np.uint32(1)) | bit_v
        u[s:s + len(idx)] = uu
        v[s:s + len(idx)] = vv
    w = weights(seed, m, wmax, wmin) if wmax > 1 else np.ones(m, dtype=np.uint32)
    return n, u, v, w


def watts_strogatz(n, k, p, seed, wmax=100, wmin=1):
    """Ring lattice with k neighbours (k even), each lattice edge (i, i+j) rewired with
    probability p to (i, x) for a uniform x (stream 11/12); rewires that would create a
    self-loop keep the lattice edge."""
    half = k // 2
    i = np.repeat(np.arange(n, dtype=np.uint64), half)
    j = np.tile(np.arange(1, half + 1, dtype=np.uint64), n)
    u = i.astype(np.uint32)
    v = ((i + j) % np.uint64(n)).astype(np.uint32)
    idx = np.arange(len(u), dtype=np.uint64)
    rew = hash64(seed, 11, idx) < _threshold(p)
    x = _uniform_int(seed, 12, idx, 0, n - 1)
    ok = rew & (x != u)
    v = np.where(ok, x, v).astype(np.uint32)
    w = weights(seed, len(u), wmax, wmin)
    return n, u, v, w


def write_graph(path, n, u, v, w, header="generated"):
    """Write the reference's edge-list format: a skipped first line, `n m`, then `u v w` lines
    (src/input/GraphInputIterator.cpp:3-36)."""
    arr = np.stack([u, v, w], axis=1).astype(np.uint64)
    with open(path, "w") as f:
        f.write("# %s\n%d %d\n" % (header, n, len(u)))
        np.savetxt(f, arr, fmt="%d")


def read_graph(path):
    """Read the reference's edge-list format (numpy; test and bench helper)."""
    with open(path) as f:
        f.readline()
        toks = f.read().split()
    n, m = int(toks[0]), int(toks[1])
    a = np.array(toks[2:2 + 3 * m], dtype=np.uint64).reshape(m, 3)
    return n, a[:, 0].astype(np.uint32), a[:, 1].astype(np.uint32), a[:, 2].astype(np.uint32)
