"""CPU tests: the oracle against the golden fixtures, and the generator."""
import hashlib
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _tiny():
    with open(os.path.join(HERE, "golden", "tiny_graphs.json")) as f:
        return json.load(f)


def _gnm():
    with open(os.path.join(HERE, "golden", "gnm_summaries.json")) as f:
        return json.load(f)


def _triples(mst):
    return sorted((int(min(a, b)), int(max(a, b)), int(w))
                  for a, b, w in zip(mst["src"], mst["dst"], mst["w"]))


@pytest.mark.parametrize("case", _tiny(), ids=lambda c: c["name"])
def test_kruskal_matches_hand_derived_forest(oracle, case):
    e = oracle.symmetric_from_undirected([tuple(t) for t in case["edges"]])
    mst, w = oracle.kruskal(e, case["n"])
    assert _triples(mst) == [tuple(t) for t in case["forest"]]
    assert w == case["weight"]


@pytest.mark.parametrize("case", _tiny(), ids=lambda c: c["name"])
def test_port_matches_hand_derived_forest(oracle, case):
    e = oracle.symmetric_from_undirected([tuple(t) for t in case["edges"]])
    mst, w, _ = oracle.boruvka_filter(e, case["n"])
    assert _triples(mst) == [tuple(t) for t in case["forest"]]
    assert w == case["weight"]


@pytest.mark.parametrize("case", _gnm(), ids=lambda c: f"n{c['n']}_m{c['m']}")
def test_gnm_summaries(oracle, case):
    e = oracle.gen_gnm(case["n"], case["m"], case["seed"], case["max_weight"])
    assert hashlib.sha256(e.tobytes()).hexdigest() == case["edges_sha256"]
    mst, w = oracle.kruskal(e, case["n"])
    assert hashlib.sha256(oracle.canon_keys(mst).tobytes()).hexdigest() == case["forest_sha256"]
    assert (len(mst), w) == (case["forest_size"], case["forest_weight"])


@pytest.mark.parametrize("n,m,seed", [(100, 150, 1), (100, 1000, 2), (5000, 12000, 3),
                                      (5000, 80000, 4), (1 << 15, 1 << 19, 5)])
def test_port_matches_kruskal(oracle, n, m, seed):
    """The restated reference filter-Boruvka yields Kruskal's canonical forest
    (exercises both the m <= 3n and the filter-recursion paths)."""
    e = oracle.gen_gnm(n, m, seed)
    a, wa = oracle.kruskal(e, n)
    b, wb, rounds = oracle.boruvka_filter(e, n)
    assert wa == wb
    assert np.array_equal(oracle.canon_keys(a), oracle.canon_keys(b))
    assert rounds > 0


def test_port_thread_counts_agree(oracle):
    e = oracle.gen_gnm(1 << 14, 1 << 17, 11)
    ref = oracle.boruvka_filter(e, 1 << 14, threads=1)
    for t in (2, 4):
        got = oracle.boruvka_filter(e, 1 << 14, threads=t)
        assert got[1] == ref[1]
        assert np.array_equal(oracle.canon_keys(got[0]), oracle.canon_keys(ref[0]))


@pytest.mark.parametrize("n,m,wmax", [(2, 1, 254), (20, 190, 254), (1000, 5000, 1),
                                      (1 << 12, 1 << 15, 254), (300, 20000, 1 << 20)])
def test_gnm_properties(oracle, n, m, wmax):
    e = oracle.gen_gnm(n, m, 7, wmax)
    assert len(e) == 2 * m
    key = (e["src"].astype(np.uint64) << np.uint64(32)) | e["dst"]
    assert np.all(np.diff(key) > 0)  # strictly (src, dst) sorted, no duplicates
    assert np.all(e["src"] != e["dst"])
    assert e["src"].max() < n and e["dst"].max() < n
    assert e["w"].min() >= 1 and e["w"].max() <= wmax
    # symmetric with equal weights
    rev = (e["dst"].astype(np.uint64) << np.uint64(32)) | e["src"]
    order = np.argsort(rev)
    assert np.array_equal(rev[order], key)
    assert np.array_equal(e["w"][order], e["w"])
    again = oracle.gen_gnm(n, m, 7, wmax)
    assert np.array_equal(again, e)


def test_gnm_rejects_too_many_edges(oracle):
    with pytest.raises(ValueError):
        oracle.gen_gnm(4, 7, 1)


def _mix64(z):
    M = (1 << 64) - 1
    z = (z + 0x9E3779B97F4A7C15) & M
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
    return z ^ (z >> 31)


def _geo_w(mode, d2, R2, wseed, j, k, wmax):
    """The generators' weight rules: hash, Euclidean, squared Euclidean."""
    import math
    if mode == 0:
        canon = (min(j, k) << 32) | max(j, k)
        return 1 + ((_mix64(wseed ^ canon) * wmax) >> 64)
    if R2 == 0:
        return 1
    if mode == 2:
        return 1 + (d2 * (wmax - 1)) // R2
    return 1 + math.isqrt((d2 * (wmax - 1) ** 2) // R2)


def _py_rgg2d(n, radius, seed, wmax=254, mode=0):
    """All-pairs restatement of the RGG-2D definition (small n only)."""
    base = _mix64(seed ^ 0x5247473244)
    wseed = _mix64(seed ^ 0x6A09E667F3BCC909)
    R = 0 if radius <= 0 else (1 << 31) if radius >= 1 else int(radius * 2147483648.0)
    cap = max(1, min(int(n ** 0.5 + 1e-9), 65536))
    while cap * cap > n:
        cap -= 1
    cap = max(cap, 1)
    G = cap if R == 0 else max(1, min((1 << 31) // R, cap))
    pts = []
    for i in range(n):
        x, y = _mix64((base + 2 * i) % (1 << 64)) >> 33, _mix64((base + 2 * i + 1) % (1 << 64)) >> 33
        cell = ((y * G) >> 31) * G + ((x * G) >> 31)
        pts.append((cell, i, x, y))
    pts.sort()
    out = []
    for j, (_, _, xj, yj) in enumerate(pts):
        for k, (_, _, xk, yk) in enumerate(pts):
            d2 = (xj - xk) ** 2 + (yj - yk) ** 2
            if k != j and d2 <= R * R:
                out.append((j, k, _geo_w(mode, d2, R * R, wseed, j, k, wmax)))
    return out


@pytest.mark.parametrize("n,radius,seed", [(1, 0.5, 1), (40, 0.2, 2), (200, 0.1, 3),
                                           (150, 1.0, 4), (90, 0.0, 5)])
def test_rgg2d_matches_definition(oracle, n, radius, seed):
    e = oracle.gen_rgg2d(n, radius, seed)
    got = [(int(a), int(b), int(w)) for a, b, w in zip(e["src"], e["dst"], e["w"])]
    assert got == _py_rgg2d(n, radius, seed)


def test_rgg2d_properties(oracle):
    n = 1 << 15
    e = oracle.gen_rgg2d(n, oracle.rgg_radius(n, 16), 7)
    s, d = e["src"].astype(np.uint64), e["dst"].astype(np.uint64)
    k = (s << np.uint64(32)) | d
    assert np.all(k[1:] > k[:-1])  # (src,dst) sorted, no duplicates
    assert np.array_equal(np.sort((d << np.uint64(32)) | s), k)  # both directions
    assert 14.0 < len(e) / n < 16.5  # border effects lower the mean degree slightly


def _py_rhg(n, gamma, k, seed, wmax=254):
    """All-pairs restatement of the RHG definition (small n only); Python's
    math module uses the same C library functions as the generators' host
    code, and Python floats round like the device code (no FMA)."""
    import math
    alpha = (gamma - 1) / 2
    xi = alpha / (alpha - 0.5)
    R = max(1.0, 2.0 * math.log(2.0 * xi * xi * n / (3.141592653589793 * k)))
    coshR, coshAR1 = math.cosh(R), math.cosh(alpha * R) - 1.0
    base = _mix64(seed ^ 0x524847)
    wseed = _mix64(seed ^ 0x6A09E667F3BCC909)
    pts = []
    for i in range(n):
        u = (_mix64((base + 2 * i) % (1 << 64)) >> 11) * 2.0 ** -53
        v = (_mix64((base + 2 * i + 1) % (1 << 64)) >> 11) * 2.0 ** -53
        r = min(R, math.acosh(1.0 + u * coshAR1) / alpha)
        theta = 6.283185307179586 * v
        band = max(0, min(15, math.floor(r * 16 / R)))
        tb = np.array([theta]).view(np.uint64)[0]
        pts.append(((band << 58) | (int(tb) >> 5), i, theta, math.exp(r), math.exp(-r),
                    math.sinh(r)))
    pts.sort(key=lambda p: (p[0], p[1]))

    def hsin(x):
        x2 = x * x
        t = 1.0 - x2 / 420.0
        for c in (342.0, 272.0, 210.0, 156.0, 110.0, 72.0, 42.0, 20.0, 6.0):
            t = 1.0 - x2 / c * t
        return x * t

    out = []
    for j in range(n):
        for q in range(n):
            if q == j:
                continue
            a, b = (pts[j], pts[q]) if j < q else (pts[q], pts[j])
            d = abs(a[2] - b[2])
            if d > 3.141592653589793:
                d = 6.283185307179586 - d
            s = hsin(d * 0.5)
            if 2.0 * s * s * a[5] * b[5] <= coshR - 0.5 * (a[3] * b[4] + a[4] * b[3]):
                canon = (min(j, q) << 32) | max(j, q)
                out.append((j, q, 1 + ((_mix64(wseed ^ canon) * wmax) >> 64)))
    return out


@pytest.mark.parametrize("n,gamma,k,seed", [(1, 3.0, 8, 1), (60, 3.0, 8, 2), (300, 3.0, 16, 3),
                                            (250, 2.6, 10, 4), (200, 4.0, 6, 5)])
def test_rhg_matches_definition(oracle, n, gamma, k, seed):
    e = oracle.gen_rhg(n, gamma, k, seed)
    got = [(int(a), int(b), int(w)) for a, b, w in zip(e["src"], e["dst"], e["w"])]
    assert got == _py_rhg(n, gamma, k, seed)


def test_rhg_properties(oracle):
    n = 1 << 15
    e = oracle.gen_rhg(n, 3.0, 16, 7)
    s, d = e["src"].astype(np.uint64), e["dst"].astype(np.uint64)
    k = (s << np.uint64(32)) | d
    assert np.all(k[1:] > k[:-1])
    assert np.array_equal(np.sort((d << np.uint64(32)) | s), k)
    deg = np.bincount(e["src"], minlength=n)
    assert 8 < len(e) / n < 32        # near the target average degree
    assert deg.max() > 20 * len(e) / n  # power law: hubs


def _weight(wseed, a, b, wmax=254):
    canon = (min(a, b) << 32) | max(a, b)
    return 1 + ((_mix64(wseed ^ canon) * wmax) >> 64)


def _py_grid(X, Y, Z, p, periodic, seed, wmax=254):
    """Set-based restatement of the lattice definition (small sizes only)."""
    pseed = _mix64(seed ^ 0x47524944)
    wseed = _mix64(seed ^ 0x6A09E667F3BCC909)
    pthr = int(p * 9007199254740992.0) if 0.0 < p < 1.0 else 0
    pairs = set()
    for z in range(Z):
        for y in range(Y):
            for x in range(X):
                v = (z * Y + y) * X + x
                for axis, side in enumerate((X, Y, Z)):
                    for step in (-1, 1):
                        c = [x, y, z]
                        t = c[axis] + step
                        if not 0 <= t < side:
                            if not periodic:
                                continue
                            t %= side
                        c[axis] = t
                        u = (c[2] * Y + c[1]) * X + c[0]
                        if u == v:
                            continue
                        canon = (min(u, v) << 32) | max(u, v)
                        if p < 1.0 and (_mix64(pseed ^ canon) >> 11) >= pthr:
                            continue
                        pairs.add((v, u))
    return [(a, b, _weight(wseed, a, b, wmax)) for a, b in sorted(pairs)]


@pytest.mark.parametrize("X,Y,Z,p,periodic", [(1, 1, 1, 1.0, True), (2, 1, 1, 1.0, True),
                                              (2, 2, 2, 1.0, True), (5, 3, 1, 1.0, False),
                                              (4, 3, 2, 1.0, True), (6, 5, 1, 0.6, True),
                                              (3, 4, 5, 0.3, False), (7, 1, 1, 1.0, True)])
def test_grid_matches_definition(oracle, X, Y, Z, p, periodic):
    e = oracle.gen_grid(X, Y, Z, p, periodic, 11)
    got = [(int(a), int(b), int(w)) for a, b, w in zip(e["src"], e["dst"], e["w"])]
    assert got == _py_grid(X, Y, Z, p, periodic, 11)


def test_grid_edge_counts():
    """Closed forms: a periodic torus with sides >= 3 is 2d-regular; the open
    box has sum over axes of (side - 1) * (other sides) edges."""
    from tests import _oracle as oracle
    assert len(oracle.gen_grid(64, 32, 1)) == 4 * 64 * 32
    assert len(oracle.gen_grid(8, 9, 10)) == 6 * 8 * 9 * 10
    assert len(oracle.gen_grid(8, 9, 10, periodic=False)) == 2 * (7 * 90 + 8 * 8 * 10 + 9 * 72)


def _py_rgg3d(n, radius, seed, wmax=254):
    """All-pairs restatement of the RGG-3D definition (small n only)."""
    base = _mix64(seed ^ 0x5247473344)
    wseed = _mix64(seed ^ 0x6A09E667F3BCC909)
    R = 0 if radius <= 0 else (1 << 31) if radius >= 1 else int(radius * 2147483648.0)
    cap = 1
    while (cap + 1) ** 3 <= n:
        cap += 1
    cap = min(cap, 1024)
    G = cap if R == 0 else max(1, min((1 << 31) // R, cap))
    M = 1 << 64
    pts = []
    for i in range(n):
        x, y, z = (_mix64((base + 3 * i + a) % M) >> 33 for a in range(3))
        cell = (((z * G) >> 31) * G + ((y * G) >> 31)) * G + ((x * G) >> 31)
        pts.append((cell, i, x, y, z))
    pts.sort()
    out = []
    for j, pj in enumerate(pts):
        for k, pk in enumerate(pts):
            if k != j and sum((pj[a] - pk[a]) ** 2 for a in (2, 3, 4)) <= R * R:
                out.append((j, k, _weight(wseed, j, k, wmax)))
    return out


@pytest.mark.parametrize("n,radius,seed", [(1, 0.5, 1), (30, 0.3, 2), (200, 0.2, 3),
                                           (64, 1.0, 4), (90, 0.0, 5)])
def test_rgg3d_matches_definition(oracle, n, radius, seed):
    e = oracle.gen_rgg3d(n, radius, seed)
    got = [(int(a), int(b), int(w)) for a, b, w in zip(e["src"], e["dst"], e["w"])]
    assert got == _py_rgg3d(n, radius, seed)


def test_rgg3d_properties(oracle):
    n = 1 << 15
    e = oracle.gen_rgg3d(n, oracle.rgg3d_radius(n, 16), 7)
    s, d = e["src"].astype(np.uint64), e["dst"].astype(np.uint64)
    k = (s << np.uint64(32)) | d
    assert np.all(k[1:] > k[:-1])
    assert np.array_equal(np.sort((d << np.uint64(32)) | s), k)
    assert 12.0 < len(e) / n < 16.5  # the cube's faces lower the mean degree


def _py_rmat(L, samples, seed, a=0.57, b=0.19, c=0.19, wmax=254):
    """Sample-by-sample restatement of the R-MAT definition."""
    import math
    base = _mix64(seed ^ 0x524D4154)
    wseed = _mix64(seed ^ 0x6A09E667F3BCC909)
    t = [min(1 << 32, math.floor(x * 4294967296.0)) for x in (a, a + b, a + b + c)]
    per = (L + 1) // 2
    pairs = set()
    for i in range(samples):
        u = v = 0
        for lvl in range(L):
            h = _mix64((base + i * per + lvl // 2) % (1 << 64))
            r = h >> 32 if lvl % 2 == 0 else h & 0xFFFFFFFF
            q = 0 if r < t[0] else 1 if r < t[1] else 2 if r < t[2] else 3
            u, v = 2 * u + (q >> 1), 2 * v + (q & 1)
        if u != v:
            pairs.add((min(u, v), max(u, v)))
    d = sorted([(x, y) for x, y in pairs] + [(y, x) for x, y in pairs])
    return [(x, y, _weight(wseed, x, y, wmax)) for x, y in d]


@pytest.mark.parametrize("L,samples,seed,abc", [(1, 10, 1, (0.57, 0.19, 0.19)),
                                                (5, 100, 2, (0.57, 0.19, 0.19)),
                                                (10, 3000, 3, (0.57, 0.19, 0.19)),
                                                (9, 2000, 4, (0.25, 0.25, 0.25)),
                                                (7, 500, 5, (0.0, 0.5, 0.5)),
                                                (6, 300, 6, (1.0, 0.0, 0.0))])
def test_rmat_matches_definition(oracle, L, samples, seed, abc):
    e = oracle.gen_rmat(L, samples, seed, *abc)
    got = [(int(x), int(y), int(w)) for x, y, w in zip(e["src"], e["dst"], e["w"])]
    assert got == _py_rmat(L, samples, seed, *abc)


def test_rmat_properties(oracle):
    e = oracle.gen_rmat(16, 1 << 19, 9)
    s, d = e["src"].astype(np.uint64), e["dst"].astype(np.uint64)
    k = (s << np.uint64(32)) | d
    assert np.all(k[1:] > k[:-1])
    assert np.array_equal(np.sort((d << np.uint64(32)) | s), k)
    deg = np.bincount(e["src"], minlength=1 << 16)
    assert deg[0] == deg.max() and deg[0] > 100 * len(e) / (1 << 16)  # hub at id 0


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("n,radius,seed,wmax", [(40, 0.3, 2, 254), (200, 0.1, 3, 7),
                                                (90, 1.0, 4, 1 << 20), (50, 0.0, 5, 254)])
def test_rgg2d_distance_weights_match_definition(oracle, mode, n, radius, seed, wmax):
    e = oracle.gen_rgg2d(n, radius, seed, wmax, distance=mode)
    got = [(int(a), int(b), int(w)) for a, b, w in zip(e["src"], e["dst"], e["w"])]
    assert got == _py_rgg2d(n, radius, seed, wmax, mode)


def test_distance_weights_follow_distance(oracle):
    """Euclidean and squared weights grow with the distance, stay in
    [1, max_weight], and agree on the edge set with the hash weights."""
    n = 1 << 12
    r = oracle.rgg_radius(n, 12)
    base = oracle.gen_rgg2d(n, r, 8)
    for mode in (1, 2):
        e = oracle.gen_rgg2d(n, r, 8, 254, distance=mode)
        assert np.array_equal(e["src"], base["src"]) and np.array_equal(e["dst"], base["dst"])
        assert e["w"].min() >= 1 and e["w"].max() <= 254
    e3 = oracle.gen_rgg3d(1 << 12, oracle.rgg3d_radius(1 << 12, 12), 8, 254, distance=1)
    assert e3["w"].min() >= 1 and e3["w"].max() <= 254
