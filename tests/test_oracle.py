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
