"""GPU parity tests: the CUDA path through the C ABI against the oracle.

Bar: bit-exact -- the forest edge set under the (w, min, max) order and its
total weight must equal the oracle's Kruskal on the same seeded input.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _tiny():
    with open(os.path.join(HERE, "golden", "tiny_graphs.json")) as f:
        return json.load(f)


def _configs(K):
    LP = K.LocalPreprocessing
    return {
        "boruvka_plain": (K.boruvka, K.AlgorithmConfig(local_preprocessing=LP.NO_PREPROCESSING)),
        "boruvka_local": (K.boruvka, K.AlgorithmConfig(local_preprocessing=LP.MODIFIED_BORUVKA)),
        "filter_boruvka": (K.filter_boruvka, K.AlgorithmConfig()),
        "filter_boruvka_t1": (K.filter_boruvka, K.AlgorithmConfig(filter_threshold=1)),
        "boruvka_dedupe": (K.boruvka, K.AlgorithmConfig(local_preprocessing=LP.NO_PREPROCESSING,
                                                        dedupe="always")),
        "filter_dedupe": (K.filter_boruvka, K.AlgorithmConfig(dedupe="always")),
    }


ALGOS = ["boruvka_plain", "boruvka_local", "filter_boruvka", "filter_boruvka_t1",
         "boruvka_dedupe", "filter_dedupe"]


def _triples(mst):
    return sorted((int(min(a, b)), int(max(a, b)), int(w))
                  for a, b, w in zip(mst["src"], mst["dst"], mst["w"]))


def _check(oracle, got, edges, n):
    ref, w = oracle.kruskal(edges, n)
    assert len(got) == len(ref)
    assert int(got["w"].astype(np.uint64).sum()) == w
    assert np.all(got["src"] < got["dst"])  # written as (min, max, w)
    assert np.array_equal(oracle.canon_keys(got), oracle.canon_keys(ref))


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("case", _tiny(), ids=lambda c: c["name"])
def test_tiny_golden(kamsta, oracle, algo, case):
    fn, cfg = _configs(kamsta)[algo]
    e = oracle.symmetric_from_undirected([tuple(t) for t in case["edges"]])
    got = fn(e, cfg, n=case["n"])
    assert _triples(got) == [tuple(t) for t in case["forest"]]


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("n,m,seed,wmax", [
    (64, 100, 1, 254), (1000, 2000, 2, 254), (1000, 20000, 3, 254), (1 << 12, 1 << 15, 4, 254),
    (1 << 16, 1 << 20, 5, 254), (1 << 16, 1 << 17, 6, 254), (1 << 14, 1 << 18, 7, 4),
    (1 << 14, 1 << 16, 8, 1), (1 << 15, 1 << 18, 9, 1 << 30), (3000, 4000000, 10, 254)])
def test_gnm_parity(kamsta, oracle, algo, n, m, seed, wmax):
    fn, cfg = _configs(kamsta)[algo]
    e = oracle.gen_gnm(n, m, seed, wmax)
    _check(oracle, fn(e, cfg, n=n), e, n)


@pytest.mark.parametrize("algo", ALGOS)
def test_isolated_and_unused_vertices(kamsta, oracle, algo):
    fn, cfg = _configs(kamsta)[algo]
    e = oracle.gen_gnm(500, 2000, 12)
    e = e.copy()
    e["src"] *= 3
    e["dst"] *= 3  # ids spread out: 2/3 of the vertices are isolated
    _check(oracle, fn(e, cfg, n=1600), e, 1600)


@pytest.mark.parametrize("algo", ALGOS)
def test_long_increasing_path(kamsta, oracle, algo):
    """Hook chains of depth n-1 (pointer jumping worst case)."""
    fn, cfg = _configs(kamsta)[algo]
    n = 1 << 16
    und = [(i, i + 1, i + 1) for i in range(n - 1)]
    e = oracle.symmetric_from_undirected(und)
    _check(oracle, fn(e, cfg, n=n), e, n)


@pytest.mark.parametrize("algo", ALGOS)
def test_star_hub(kamsta, oracle, algo):
    """One vertex adjacent to all others (segmented minimum over a hub)."""
    fn, cfg = _configs(kamsta)[algo]
    n = 1 << 17
    rng = np.random.default_rng(3)
    w = rng.integers(1, 255, n - 1)
    und = [(0, i, int(w[i - 1])) for i in range(1, n)] + [(i, i + 1, 200) for i in range(1, n - 1)]
    e = oracle.symmetric_from_undirected(und)
    _check(oracle, fn(e, cfg, n=n), e, n)


@pytest.mark.parametrize("algo", ALGOS)
def test_disconnected_components(kamsta, oracle, algo):
    fn, cfg = _configs(kamsta)[algo]
    parts = []
    off = 0
    for k, (n, m) in enumerate([(300, 900), (2000, 3000), (1, 0), (5000, 60000), (2, 1)]):
        if m:
            g = oracle.gen_gnm(n, m, 20 + k)
            g = g.copy()
            g["src"] += off
            g["dst"] += off
            parts.append(g)
        off += n
    e = np.concatenate(parts)
    _check(oracle, fn(e, cfg, n=off), e, off)


def test_empty_inputs(kamsta):
    empty = np.zeros(0, kamsta.WEDGE)
    assert len(kamsta.boruvka(empty, n=0)) == 0
    assert len(kamsta.boruvka(empty, n=10)) == 0


def test_validation_rejects_unsorted_and_out_of_range(kamsta, oracle):
    e = oracle.gen_gnm(100, 300, 1)
    cfg = kamsta.AlgorithmConfig(validate=True)
    bad = e.copy()
    bad[[5, 6]] = bad[[6, 5]]
    with pytest.raises(kamsta.KamstaError) as ei:
        kamsta.boruvka(bad, cfg, n=100)
    assert ei.value.status == 1
    with pytest.raises(kamsta.KamstaError) as ei:
        kamsta.boruvka(e, cfg, n=50)
    assert ei.value.status == 1
    # the context stays usable after a rejected call
    _check(oracle, kamsta.boruvka(e, cfg, n=100), e, 100)


def test_memory_limit_fails_cleanly(kamsta, oracle):
    """A context over its memory limit fails with E_OOM, before any device
    memory is taken or in the middle of a solve, and stays usable."""
    import torch
    n = 1 << 16
    e = oracle.gen_gnm(n, 1 << 20, 21)
    d = torch.from_numpy(e.view(np.uint32).reshape(-1, 3).view(np.int32)).cuda()
    out = torch.empty((n, 3), dtype=torch.int32, device="cuda")
    ctx = kamsta.Context(0)

    def solve():
        k = ctx.boruvka_dev(d.data_ptr(), len(e), n, out.data_ptr())
        return out[:k].cpu().numpy().view(np.uint32).reshape(-1).view(kamsta.WEDGE)

    ctx.set_memory_limit(1 << 20)  # below the vertex arrays alone
    with pytest.raises(kamsta.KamstaError) as ei:
        solve()
    assert ei.value.status == kamsta._native.E_OOM
    ctx.set_memory_limit(0)
    _check(oracle, solve(), e, n)
    # the vertex arrays stay reserved, so now the edge lists go over
    ctx.set_memory_limit(1 << 20)
    with pytest.raises(kamsta.KamstaError) as ei:
        solve()
    assert ei.value.status == kamsta._native.E_OOM
    ctx.set_memory_limit(0)
    _check(oracle, solve(), e, n)
    ctx.close()


def test_validation_across_input_pieces(kamsta, oracle):
    """The host entry point copies the input in 16 pieces and starts the
    first pass on each as it lands; validation must still compare every
    entry with its predecessor, including across pieces and CTA chunks."""
    n = 1 << 18
    e = oracle.gen_gnm(n, 1 << 22, 33)
    cfg = kamsta.AlgorithmConfig(validate=True)
    _check(oracle, kamsta.boruvka(e, cfg, n=n), e, n)
    per = (len(e) + 15) // 16
    for at in (per, 7 * per, len(e) // 2):  # piece boundaries and a mid point
        bad = e.copy()
        bad[[at - 1, at]] = bad[[at, at - 1]]
        with pytest.raises(kamsta.KamstaError) as ei:
            kamsta.boruvka(bad, cfg, n=n)
        assert ei.value.status == 1


def test_wedge64_entry_point(kamsta, oracle):
    e = oracle.gen_gnm(2000, 10000, 31)
    e64 = np.zeros(len(e), kamsta.WEDGE64)
    e64["src"], e64["dst"], e64["w"] = e["src"], e["dst"], e["w"]
    got = kamsta.boruvka_wedge64(e64, n=2000)
    ref, w = oracle.kruskal(e, 2000)
    assert int(got["w"].sum()) == w
    a = (got["src"].astype(np.uint64) << np.uint64(32)) | got["dst"]
    assert np.array_equal(np.sort(a), oracle.canon_keys(ref))


def test_sort_output_flag(kamsta, oracle):
    e = oracle.gen_gnm(4000, 40000, 32)
    got = kamsta.boruvka(e, kamsta.AlgorithmConfig(sort_output=True), n=4000)
    key = (got["src"].astype(np.uint64) << np.uint64(32)) | got["dst"]
    assert np.all(np.diff(key) > 0)


def test_device_entry_point_and_generator(kamsta, oracle):
    import torch
    n, m, seed = 1 << 15, 1 << 18, 77
    ctx = kamsta.Context(0)
    d = torch.empty((2 * m, 3), dtype=torch.int32, device="cuda")
    assert ctx.gen_gnm_dev(n, m, seed, 254, d.data_ptr()) == 2 * m
    torch.cuda.synchronize()
    host = d.cpu().numpy().view(np.uint32).reshape(-1).view(kamsta.WEDGE)
    ref_edges = oracle.gen_gnm(n, m, seed)
    assert np.array_equal(host, ref_edges)  # device generator == oracle generator
    out = torch.empty((n, 3), dtype=torch.int32, device="cuda")
    stats = {}
    k = ctx.boruvka_dev(d.data_ptr(), 2 * m, n, out.data_ptr(),
                        kamsta.AlgorithmConfig(local_preprocessing=1),
                        stream=torch.cuda.current_stream().cuda_stream, stats=stats)
    got = out[:k].cpu().numpy().view(np.uint32).reshape(-1).view(kamsta.WEDGE)
    _check(oracle, got, ref_edges, n)
    assert stats["gpu_launches"] > 0 and stats["device_ms"] > 0
    ctx.close()


@pytest.mark.parametrize("n,m", [(1 << 10, 1 << 14), (1 << 20, 1 << 24)])
def test_device_generator_matches_oracle(kamsta, oracle, n, m):
    import torch
    ctx = kamsta.Context(0)
    d = torch.empty((2 * m, 3), dtype=torch.int32, device="cuda")
    ctx.gen_gnm_dev(n, m, 5, 254, d.data_ptr())
    torch.cuda.synchronize()
    host = d.cpu().numpy().view(np.uint32).reshape(-1).view(kamsta.WEDGE)
    assert np.array_equal(host, oracle.gen_gnm(n, m, 5))


@pytest.mark.parametrize("algo", ["boruvka_plain", "boruvka_local", "filter_boruvka"])
def test_exactness_n22_m26(kamsta, oracle, algo):
    """The bit-exact check size of the large configuration: G(n=2^22, m=2^26)."""
    fn, cfg = _configs(kamsta)[algo]
    n, m = 1 << 22, 1 << 26
    e = oracle.gen_gnm(n, m, 2026)
    _check(oracle, fn(e, cfg, n=n), e, n)


@pytest.mark.parametrize("mode,ratio", [("always", 0), ("auto", 2), ("auto", 8)])
def test_dedupe_runs_and_keeps_the_forest(kamsta, oracle, mode, ratio):
    """Parallel-edge removal (radix sort + keep the lightest) leaves the
    forest unchanged and actually runs on a graph whose contraction creates
    many parallel edges."""
    n, m = 1 << 14, 1 << 19
    e = oracle.gen_gnm(n, m, 31, 254)
    st = {}
    cfg = kamsta.AlgorithmConfig(dedupe=mode, dedupe_ratio=ratio)
    got = kamsta.boruvka(e, cfg, n=n, stats=st)
    _check(oracle, got, e, n)
    assert st["dedupe_passes"] > 0
    st0 = {}
    kamsta.boruvka(e, kamsta.AlgorithmConfig(dedupe="never", dedupe_ratio=ratio), n=n, stats=st0)
    assert st0["dedupe_passes"] == 0


def test_row_scan_contraction_is_used_and_exact(kamsta, oracle):
    """The heaviest class of a dense G(n,m) is contracted by scanning only the
    rows of the few vertices outside the giant component; the forest stays
    the oracle's."""
    n, m = 1 << 20, 1 << 24
    e = oracle.gen_gnm(n, m, 77)
    st = {}
    got = kamsta.boruvka(e, kamsta.AlgorithmConfig(local_preprocessing=1), n=n, stats=st)
    _check(oracle, got, e, n)
    assert st["row_scans"] >= 1


@pytest.mark.parametrize("items,seg", [(8, 8), (12, 4), (6, 2), (8, 4)])
def test_tile_sizes_agree(kamsta, oracle, items, seg):
    """The tiles (entries / records per thread) change the schedule only."""
    n, m = 1 << 18, 1 << 22
    e = oracle.gen_gnm(n, m, 91)
    for lp in (0, 1):
        cfg = kamsta.AlgorithmConfig(local_preprocessing=lp, items_per_thread=items,
                                     seg_items_per_thread=seg)
        _check(oracle, kamsta.boruvka(e, cfg, n=n), e, n)
        _check(oracle, kamsta.filter_boruvka(e, cfg, n=n), e, n)


def _disjoint_dense(kamsta, comps, size, seed, wmax):
    """`comps` disjoint complete graphs of `size` vertices, weights U[1, wmax],
    both directions, (src, dst)-sorted: every component contracts to one
    vertex within a few rounds while most of its edges are still listed."""
    rng = np.random.default_rng(seed)
    iu, ju = np.triu_indices(size, 1)
    base = (np.arange(comps, dtype=np.int64) * size)[:, None]
    u = (base + iu[None, :]).ravel()
    v = (base + ju[None, :]).ravel()
    w = rng.integers(1, wmax + 1, len(u))
    s, d, ww = np.concatenate([u, v]), np.concatenate([v, u]), np.concatenate([w, w])
    order = np.lexsort((d, s))
    e = np.empty(len(s), kamsta.WEDGE)
    e["src"], e["dst"], e["w"] = s[order], d[order], ww[order]
    return e, comps * size


@pytest.mark.parametrize("algo", ["boruvka_plain", "boruvka_local", "filter_boruvka",
                                  "filter_boruvka_t1"])
@pytest.mark.parametrize("case", ["gnm_dense", "gnm_large", "cliques", "cliques_ties", "rhg",
                                  "rmat"])
def test_parallel_edge_heavy_graphs(kamsta, oracle, algo, case):
    """Graphs whose contraction leaves many parallel edges between few
    components (dense G(n,m), disjoint cliques with and without weight ties,
    hubs) give the oracle's forest."""
    fn, cfg = _configs(kamsta)[algo]
    if case == "gnm_dense":
        n = 1 << 14
        e = oracle.gen_gnm(n, 1 << 21, 41)
    elif case == "gnm_large":
        n = 1 << 20
        e = oracle.gen_gnm(n, 1 << 24, 42)
    elif case == "cliques":
        e, n = _disjoint_dense(kamsta, 2048, 48, 43, 254)
    elif case == "cliques_ties":
        e, n = _disjoint_dense(kamsta, 1024, 64, 44, 3)
    elif case == "rhg":
        n = 1 << 18
        e = oracle.gen_rhg(n, 2.6, 32.0, 45)
    else:
        n = 1 << 18
        e = oracle.gen_rmat(18, 1 << 23, 46)
    _check(oracle, fn(e, cfg, n=n), e, n)


def _clique_path(kamsta, k, size, links, seed):
    """k cliques of `size` vertices (weight 5) on a path, neighbours joined
    by `links` distinct random vertex pairs of weights U[6, 254].  The
    cliques contract first; the heavier class then starts with k vertices
    and about k * links parallel records, most of which die within two
    rounds as the path contracts."""
    rng = np.random.default_rng(seed)
    iu, ju = np.triu_indices(size, 1)
    base = (np.arange(k, dtype=np.int64) * size)[:, None]
    u = [(base + iu[None, :]).ravel()]
    v = [(base + ju[None, :]).ravel()]
    w = [np.full(u[0].shape, 5)]
    for c in range(k - 1):
        pairs = rng.choice(size * size, links, replace=False)
        u.append(c * size + pairs // size)
        v.append((c + 1) * size + pairs % size)
        w.append(rng.integers(6, 255, links))
    u, v, w = np.concatenate(u), np.concatenate(v), np.concatenate(w)
    s, d, ww = np.concatenate([u, v]), np.concatenate([v, u]), np.concatenate([w, w])
    order = np.lexsort((d, s))
    e = np.empty(len(s), kamsta.WEDGE)
    e["src"], e["dst"], e["w"] = s[order], d[order], ww[order]
    return e, k * size


@pytest.mark.parametrize("algo", ["boruvka_plain", "boruvka_local", "filter_boruvka"])
def test_clique_path(kamsta, oracle, algo):
    """Tied clique weights, then a path of heavy multi-links: the forest
    stays the oracle's (the (w, min, max) order decides the ties)."""
    fn, cfg = _configs(kamsta)[algo]
    e, n = _clique_path(kamsta, 1024, 32, 256, 47)
    _check(oracle, fn(e, cfg, n=n), e, n)


_REF_CASES = {
    "gnm_2e16_2e20": lambda O: (O.gen_gnm(1 << 16, 1 << 20, 2026), 1 << 16),
    "gnm_2e22_2e26": lambda O: (O.gen_gnm(1 << 22, 1 << 26, 2026), 1 << 22),
    "gnm_ties_w4": lambda O: (O.gen_gnm(1 << 18, 1 << 21, 31, 4), 1 << 18),
    "rgg2d_2e20": lambda O: (O.gen_rgg2d(1 << 20, O.rgg_radius(1 << 20, 16), 32), 1 << 20),
    "rhg_2e20": lambda O: (O.gen_rhg(1 << 20, 3.0, 16, 33), 1 << 20),
}


@pytest.mark.parametrize("algo", ["boruvka_plain", "boruvka_local", "filter_boruvka"])
@pytest.mark.parametrize("case", list(_REF_CASES))
def test_gpu_equals_reference_code(kamsta, oracle, algo, case):
    """The GPU forest against the REFERENCE'S OWN code on the same input
    (oracle/_ref, KaMSTa's local filter-Boruvka built from its sources):
    bit-identical edge set to its all-local run, and the same total weight
    as its single-rank preprocessing path."""
    if not oracle.ref_available():
        pytest.skip("the reference build is not present")
    fn, cfg = _configs(kamsta)[algo]
    e, n = _REF_CASES[case](oracle)
    got = fn(e, cfg, n=n)
    ref, ref_w, _ = oracle.ref_all_local(e, n)
    assert int(got["w"].astype(np.uint64).sum()) == ref_w
    assert np.array_equal(oracle.canon_keys(got), oracle.canon_keys(ref))
    _, w1, _ = oracle.ref_local_contraction(e, n)
    assert w1 == ref_w


def test_tile_autotuner_in_the_library(kamsta, oracle):
    """kamsta_autotune_tiles times every tile pair on the input, keeps the
    fastest in the context, and later solves with default tiles use it and
    give the same forest."""
    import torch
    n, m = 1 << 18, 1 << 22
    e = oracle.gen_gnm(n, m, 61)
    ctx = kamsta.Context(0)
    d = torch.from_numpy(e.view(np.uint32).reshape(-1, 3).view(np.int32)).cuda()
    o = torch.empty((n, 3), dtype=torch.int32, device="cuda")
    t = ctx.autotune_tiles(d.data_ptr(), len(e), n, o.data_ptr())
    assert (t["items_per_thread"], t["seg_items_per_thread"]) in [(6, 2), (8, 2), (12, 2),
                                                                  (6, 4), (8, 4), (12, 4)]
    assert all(v > 0 for v in t["ms"].values())
    key = f'{t["items_per_thread"]}x{t["seg_items_per_thread"]}'
    assert t["ms"][key] == min(t["ms"].values())
    k = ctx.boruvka_dev(d.data_ptr(), len(e), n, o.data_ptr())
    got = o[:k].cpu().numpy().view(np.uint32).reshape(-1).view(kamsta.WEDGE)
    _check(oracle, got, e, n)
    ctx.set_tiles(12, 4)
    with pytest.raises(kamsta.KamstaError):
        ctx.set_tiles(7, 2)
    ctx.close()
