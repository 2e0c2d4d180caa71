"""CPU tests: the reference's OWN code against the oracle.

oracle/_ref/libkamsta_ref.so is KaMSTa's single-rank local filter-Boruvka
(local_mst_respecting_cut_edges.hpp:262-302 driven as local_contraction.hpp:
114-150 drives it) compiled from the reference's sources against the
oracle's single-rank shims (oracle/ref_build.py).  These tests pin the
oracle to it:
  * its MSF weight equals Kruskal's (and the hand-derived golden answers);
  * with every vertex local, its forest is bit-for-bit Kruskal's canonical
    (w, min, max) forest and the port's (oracle.cpp's restatement);
  * in the true single-rank mode (first and last vertex are cut vertices,
    compared by weight only, mst_utils_cut_edges.hpp:129-146) the edge set
    may leave the canonical forest only under weight ties, never the weight.
"""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def ref(oracle):
    if not oracle.ref_available():
        pytest.skip("the reference's sources (or their amalgam) are not present")
    oracle.ref_lib()
    return oracle


def _triples(mst):
    return sorted((int(min(a, b)), int(max(a, b)), int(w))
                  for a, b, w in zip(mst["src"], mst["dst"], mst["w"]))


def _tiny():
    with open(os.path.join(HERE, "golden", "tiny_graphs.json")) as f:
        return [c for c in json.load(f) if all(e[2] <= 255 for e in c["edges"])]


@pytest.mark.parametrize("case", _tiny(), ids=lambda c: c["name"])
def test_reference_code_on_golden_graphs(ref, case):
    e = ref.symmetric_from_undirected([tuple(t) for t in case["edges"]])
    forest, w, _ = ref.ref_all_local(e, case["n"])
    assert _triples(forest) == [tuple(t) for t in case["forest"]]
    assert w == case["weight"]
    _, w1, _ = ref.ref_local_contraction(e, case["n"])
    assert w1 == case["weight"]


def _graphs(oracle):
    n = 1 << 16
    return [
        ("gnm_2e16_2e20", oracle.gen_gnm(n, 1 << 20, 2026), n),     # the CPU-runnable config
        ("gnm_ties_w4", oracle.gen_gnm(1 << 15, 1 << 19, 7, 4), 1 << 15),
        ("gnm_sparse_isolated", oracle.gen_gnm(1 << 16, 20000, 8), 1 << 16),
        ("rgg2d", oracle.gen_rgg2d(n, oracle.rgg_radius(n, 16), 9), n),
        ("rhg", oracle.gen_rhg(n, 3.0, 16, 10), n),
        ("grid_ties", oracle.gen_grid(256, 256, 1, 1.0, True, 11, 3), 256 * 256),
    ]


@pytest.mark.parametrize("idx", range(6))
def test_reference_code_equals_kruskal_and_port(ref, idx):
    name, e, n = _graphs(ref)[idx]
    kr, kw = ref.kruskal(e, n)
    # every vertex local: the reference's rounds give the canonical forest
    a, aw, ainfo = ref.ref_all_local(e, n)
    assert aw == kw, name
    assert ainfo["finish_edges"] == 0
    assert np.array_equal(ref.canon_keys(a), ref.canon_keys(kr)), name
    p, pw, _ = ref.boruvka_filter(e, n)
    assert pw == kw and np.array_equal(ref.canon_keys(p), ref.canon_keys(a)), name
    # the reference's single-rank preprocessing: the weight always
    b, bw, binfo = ref.ref_local_contraction(e, n)
    assert bw == kw, name
    assert len(b) == len(kr)
    assert binfo["local_forest_edges"] > 0.99 * len(kr) or len(kr) < 100
    if name in ("gnm_2e16_2e20", "gnm_sparse_isolated"):
        # weights 1..254 and low degrees at vertex 0 and n-1: no tie there
        assert np.array_equal(ref.canon_keys(b), ref.canon_keys(kr)), name
    else:
        # ties at a cut vertex (RHG's vertex 0 is a hub; grid and w<=4 are
        # all ties) may swap equal-weight edges, a handful at most
        diff = np.setdiff1d(ref.canon_keys(b), ref.canon_keys(kr))
        assert len(diff) <= max(16, len(kr) // 1000), (name, len(diff))


def test_reference_build_rejects_wide_weights(ref):
    e = ref.gen_gnm(100, 300, 1, 1 << 20)
    with pytest.raises(ValueError):
        ref.ref_all_local(e, 100)
