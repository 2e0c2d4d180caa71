"""ctypes access to the oracle (oracle/liboracle.so) for the tests.

The oracle is test infrastructure: it checks the GPU results and is never
part of the product path.
"""
import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
from oracle import build as _build  # noqa: E402

WEDGE = np.dtype([("src", "<u4"), ("dst", "<u4"), ("w", "<u4")])
_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(_build.build())
        P, U32, U64 = C.c_void_p, C.c_uint32, C.c_uint64
        L.oracle_kruskal.argtypes = [P, U64, U32, P, C.POINTER(U64), C.POINTER(U64)]
        L.oracle_boruvka_filter.argtypes = [P, U64, U32, C.c_int, P, C.POINTER(U64),
                                            C.POINTER(U64), C.POINTER(U32)]
        L.oracle_gen_gnm.argtypes = [U32, U64, U64, U32, P, C.POINTER(U64)]
        L.oracle_gen_rgg2d.argtypes = [U32, C.c_double, U64, U32, U32, P, U64, C.POINTER(U64)]
        L.oracle_gen_rhg.argtypes = [U32, C.c_double, C.c_double, U64, U32, P, U64,
                                     C.POINTER(U64)]
        L.oracle_gen_grid.argtypes = [U32, U32, U32, C.c_double, C.c_int, U64, U32, P, U64,
                                      C.POINTER(U64)]
        L.oracle_gen_rgg3d.argtypes = [U32, C.c_double, U64, U32, U32, P, U64, C.POINTER(U64)]
        L.oracle_gen_rmat.argtypes = [U32, U64, C.c_double, C.c_double, C.c_double, U64, U32, P,
                                      U64, C.POINTER(U64)]
        L.oracle_max_threads.restype = C.c_int
        _lib = L
    return _lib


def gen_gnm(n: int, m: int, seed: int, max_weight: int = 254) -> np.ndarray:
    out = np.empty(max(2 * m, 1), WEDGE)
    cnt = C.c_uint64()
    rc = lib().oracle_gen_gnm(n, m, seed, max_weight, out.ctypes.data, C.byref(cnt))
    if rc != 0:
        raise ValueError("oracle_gen_gnm: m exceeds n(n-1)/2")
    return out[: cnt.value]


def gen_rgg2d(n: int, radius: float, seed: int, max_weight: int = 254,
              distance: int = 0) -> np.ndarray:
    cnt = C.c_uint64()
    rc = lib().oracle_gen_rgg2d(n, radius, seed, max_weight, distance, None, 0, C.byref(cnt))
    if rc not in (0, 2):
        raise ValueError("oracle_gen_rgg2d: bad arguments")
    out = np.empty(max(cnt.value, 1), WEDGE)
    rc = lib().oracle_gen_rgg2d(n, radius, seed, max_weight, distance, out.ctypes.data,
                                cnt.value, C.byref(cnt))
    assert rc == 0
    return out[: cnt.value]


def gen_rhg(n: int, gamma: float, avg_degree: float, seed: int,
            max_weight: int = 254) -> np.ndarray:
    cnt = C.c_uint64()
    rc = lib().oracle_gen_rhg(n, gamma, avg_degree, seed, max_weight, None, 0, C.byref(cnt))
    if rc not in (0, 2):
        raise ValueError("oracle_gen_rhg: bad arguments")
    out = np.empty(max(cnt.value, 1), WEDGE)
    rc = lib().oracle_gen_rhg(n, gamma, avg_degree, seed, max_weight, out.ctypes.data,
                              cnt.value, C.byref(cnt))
    assert rc == 0
    return out[: cnt.value]


def _counted(fn, *args):
    """Runs a count-then-write oracle generator: a counting call, then the
    write into an array of that size."""
    cnt = C.c_uint64()
    rc = fn(*args, None, 0, C.byref(cnt))
    if rc not in (0, 2):
        raise ValueError(f"{fn.__name__}: bad arguments")
    out = np.empty(max(cnt.value, 1), WEDGE)
    rc = fn(*args, out.ctypes.data, cnt.value, C.byref(cnt))
    assert rc == 0
    return out[: cnt.value]


def gen_grid(x: int, y: int, z: int = 1, p: float = 1.0, periodic: bool = True, seed: int = 1,
             max_weight: int = 254) -> np.ndarray:
    return _counted(lib().oracle_gen_grid, x, y, z, p, int(periodic), seed, max_weight)


def gen_rgg3d(n: int, radius: float, seed: int, max_weight: int = 254,
              distance: int = 0) -> np.ndarray:
    return _counted(lib().oracle_gen_rgg3d, n, radius, seed, max_weight, distance)


def gen_rmat(log_n: int, samples: int, seed: int, a: float = 0.57, b: float = 0.19,
             c: float = 0.19, max_weight: int = 254) -> np.ndarray:
    return _counted(lib().oracle_gen_rmat, log_n, samples, a, b, c, seed, max_weight)


def rgg3d_radius(n: int, avg_degree: float) -> float:
    """Radius giving an expected degree `avg_degree` away from the border."""
    import math
    return (3.0 * avg_degree / (4.0 * math.pi * n)) ** (1.0 / 3.0)


def rgg_radius(n: int, avg_degree: float) -> float:
    """Radius giving an expected degree `avg_degree` away from the border."""
    import math
    return math.sqrt(avg_degree / (math.pi * n))


def kruskal(edges: np.ndarray, n: int):
    e = np.ascontiguousarray(edges, dtype=WEDGE)
    out = np.empty(max(n, 1), WEDGE)
    cnt, w = C.c_uint64(), C.c_uint64()
    rc = lib().oracle_kruskal(e.ctypes.data, len(e), n, out.ctypes.data, C.byref(cnt), C.byref(w))
    assert rc == 0
    return out[: cnt.value].copy(), int(w.value)


def boruvka_filter(edges: np.ndarray, n: int, threads: int = 0):
    """Restated reference local filter-Boruvka (timed CPU baseline)."""
    e = np.ascontiguousarray(edges, dtype=WEDGE)
    out = np.empty(max(n, 1), WEDGE)
    cnt, w, r = C.c_uint64(), C.c_uint64(), C.c_uint32()
    rc = lib().oracle_boruvka_filter(e.ctypes.data, len(e), n, threads, out.ctypes.data,
                                     C.byref(cnt), C.byref(w), C.byref(r))
    assert rc == 0
    return out[: cnt.value].copy(), int(w.value), int(r.value)


_ref = None


def ref_available() -> bool:
    from oracle import ref_build
    return ref_build.available()


def ref_lib():
    """The reference's own single-rank local filter-Boruvka, compiled from its
    sources with the oracle's shims (oracle/ref_build.py)."""
    global _ref
    if _ref is None:
        from oracle import ref_build
        L = C.CDLL(ref_build.build())
        P, U64 = C.c_void_p, C.c_uint64
        for f in (L.ref_local_contraction, L.ref_boruvka_filter_all_local):
            f.argtypes = [P, U64, C.c_int, P, C.POINTER(U64), C.POINTER(U64),
                          C.POINTER(C.c_double)]
        L.ref_set_input.argtypes = [P, U64]
        L.ref_run.argtypes = [C.c_int, C.c_int, P, C.POINTER(U64), C.POINTER(U64),
                              C.POINTER(C.c_double)]
        L.ref_max_threads.restype = C.c_int
        _ref = L
    return _ref


def _ref_call(fn, edges, n, threads):
    e = np.ascontiguousarray(edges, dtype=WEDGE)
    out = np.empty(max(n, 1), WEDGE)
    cnt, w, info = C.c_uint64(), C.c_uint64(), (C.c_double * 4)()
    rc = fn(e.ctypes.data, len(e), threads, out.ctypes.data, C.byref(cnt), C.byref(w), info)
    if rc == 2:
        raise ValueError("reference build: weights must be <= 255 (WEdge_4_1)")
    assert rc == 0
    return out[: cnt.value].copy(), int(w.value), {
        "local_forest_edges": int(info[0]), "finish_edges": int(info[1]),
        "reference_s": info[2], "finish_s": info[3]}


class RefSession:
    """Repeated runs of the reference build on one input: the input's
    std::vector<WEdge> copy is made once (the reference benchmark builds it
    before its timer starts, benchmarks/mst.cpp:198-212)."""

    def __init__(self, edges: np.ndarray, n: int):
        self.e = np.ascontiguousarray(edges, dtype=WEDGE)
        self.n = n
        rc = ref_lib().ref_set_input(self.e.ctypes.data, len(self.e))
        if rc == 2:
            raise ValueError("reference build: weights must be <= 255 (WEdge_4_1)")
        self.out = np.empty(max(n, 1), WEDGE)

    def run(self, all_local: bool = False, threads: int = 0):
        cnt, w, info = C.c_uint64(), C.c_uint64(), (C.c_double * 4)()
        rc = ref_lib().ref_run(threads, int(all_local), self.out.ctypes.data, C.byref(cnt),
                               C.byref(w), info)
        assert rc == 0
        return self.out[: cnt.value], int(w.value), {
            "local_forest_edges": int(info[0]), "finish_edges": int(info[1]),
            "reference_s": info[2], "finish_s": info[3]}

    def close(self):
        ref_lib().ref_clear_input()


def ref_local_contraction(edges: np.ndarray, n: int, threads: int = 0):
    """The reference's single-rank MODIFIED_BORUVKA preprocessing (first and
    last vertex are cut vertices), the few edges it leaves finished by
    Kruskal: (forest, weight, info)."""
    return _ref_call(ref_lib().ref_local_contraction, edges, n, threads)


def ref_all_local(edges: np.ndarray, n: int, threads: int = 0):
    """The reference's boruvka_filter with every vertex local: the whole
    forest from the reference's own rounds."""
    return _ref_call(ref_lib().ref_boruvka_filter_all_local, edges, n, threads)


def canon_keys(mst: np.ndarray) -> np.ndarray:
    """Sorted (min << 32 | max) keys of a forest: order-free edge-set identity."""
    a = np.minimum(mst["src"], mst["dst"]).astype(np.uint64)
    b = np.maximum(mst["src"], mst["dst"]).astype(np.uint64)
    return np.sort((a << np.uint64(32)) | b)


def symmetric_from_undirected(und, n=None) -> np.ndarray:
    """Both directions, sorted by (src, dst), from (u, v, w) triples."""
    und = list(und)
    rows = []
    for u, v, w in und:
        rows.append((u, v, w))
        rows.append((v, u, w))
    rows.sort(key=lambda t: (t[0], t[1]))
    out = np.empty(len(rows), WEDGE)
    for i, (u, v, w) in enumerate(rows):
        out[i] = (u, v, w)
    return out


def py_kruskal(edges: np.ndarray, n: int):
    """Independent pure-Python Kruskal under (w, src, dst) over all entries
    (base_case_mst_algos.hpp:91-112), for small cases."""
    order = sorted(range(len(edges)), key=lambda i: (int(edges["w"][i]), int(edges["src"][i]),
                                                    int(edges["dst"][i])))
    parent = list(range(n))

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    res = []
    for i in order:
        a, b = find(int(edges["src"][i])), find(int(edges["dst"][i]))
        if a == b:
            continue
        parent[a] = b
        res.append((int(edges["src"][i]), int(edges["dst"][i]), int(edges["w"][i])))
    return res
