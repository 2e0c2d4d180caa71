"""Batched solve (kamsta_mst_batch / kamsta_mst_batch_dev) against the oracle.

Each graph of a batch must give exactly the forest it gives alone: the
oracle's Kruskal edge set and weight, written (min, max, w) and sorted by
(src, dst); a malformed graph is reported on its own descriptor and leaves
the others untouched.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sorted_ref(oracle, e, n):
    ref, w = oracle.kruskal(e, n)
    t = np.empty(len(ref), ref.dtype)
    lo = np.minimum(ref["src"], ref["dst"])
    hi = np.maximum(ref["src"], ref["dst"])
    order = np.lexsort((hi, lo))
    t["src"], t["dst"], t["w"] = lo[order], hi[order], ref["w"][order]
    return t, w


def _mixed_graphs(oracle, count, seed):
    rng = np.random.default_rng(seed)
    graphs = []
    for i in range(count):
        kind = i % 5
        if kind == 0:
            n = int(rng.integers(2, 40))
            m = int(rng.integers(0, n * (n - 1) // 2 + 1))
        else:
            n = int(2 ** rng.uniform(6, 14))
            m = min(n * (n - 1) // 2, int(n * rng.uniform(2, 16)))
        wmax = [254, 254, 4, 1, 1 << 20][i % 5]
        e = oracle.gen_gnm(n, m, seed * 1000 + i, wmax) if m else np.empty(0, oracle_wedge())
        graphs.append((e, n))
    return graphs


def oracle_wedge():
    from kamsta_gb300 import WEDGE
    return WEDGE


def test_batch_host_matches_oracle(kamsta, oracle):
    graphs = _mixed_graphs(oracle, 60, 3)
    graphs += [(np.empty(0, kamsta.WEDGE), 0), (np.empty(0, kamsta.WEDGE), 1),
               (np.empty(0, kamsta.WEDGE), 7)]
    st = {}
    res = kamsta.batch(graphs, kamsta.AlgorithmConfig(
        local_preprocessing=kamsta.LocalPreprocessing.MODIFIED_BORUVKA), stats=st)
    assert st["graphs"] == len(graphs) and st["waves"] >= 1
    for (e, n), (status, got) in zip(graphs, res):
        assert status == 0
        ref, w = _sorted_ref(oracle, e, n)
        assert np.array_equal(got, ref)
        assert int(got["w"].astype(np.uint64).sum()) == w


@pytest.mark.parametrize("lp,filt", [(0, False), (1, False), (0, True)])
def test_batch_small_budget_many_waves(kamsta, oracle, lp, filt):
    graphs = _mixed_graphs(oracle, 40, 11 + lp)
    cfg = kamsta.AlgorithmConfig(local_preprocessing=lp, filter=filt)
    st = {}
    res = kamsta.batch(graphs, cfg, budget_bytes=1 << 20, stats=st)
    assert st["waves"] > 5
    for (e, n), (status, got) in zip(graphs, res):
        assert status == 0
        ref, _ = _sorted_ref(oracle, e, n)
        assert np.array_equal(got, ref)


def test_batch_bad_graph_is_isolated(kamsta, oracle):
    graphs = _mixed_graphs(oracle, 12, 5)
    bad = graphs[4][0].copy()
    bad["dst"][len(bad) // 2] = graphs[4][1] + 3  # id >= n
    graphs[4] = (bad, graphs[4][1])
    unsorted = graphs[7][0][::-1].copy()
    graphs[7] = (unsorted, graphs[7][1])
    res = kamsta.batch(graphs, kamsta.AlgorithmConfig(validate=True))
    for i, ((e, n), (status, got)) in enumerate(zip(graphs, res)):
        if i in (4, 7):
            assert status == kamsta._native.E_INPUT
            assert len(got) == 0
        else:
            assert status == 0
            ref, _ = _sorted_ref(oracle, e, n)
            assert np.array_equal(got, ref)


def test_batch_dev_equals_alone(kamsta):
    """Device batch == each graph solved alone by kamsta_mst_boruvka_dev."""
    import torch
    ctx = kamsta.Context(0)
    rng = np.random.default_rng(7)
    specs = [(int(2 ** rng.uniform(8, 16)), float(rng.uniform(2, 16))) for _ in range(48)]
    specs.append((1 << 18, 8.0))
    bufs, outs, descs = [], [], (kamsta.GraphDesc * len(specs))()
    for i, (n, deg) in enumerate(specs):
        m = min(n * (n - 1) // 2, int(n * deg / 2))
        d = torch.empty((2 * m, 3), dtype=torch.int32, device="cuda")
        md = ctx.gen_gnm_dev(n, m, 100 + i, 254, d.data_ptr())
        o = torch.zeros((max(n, 1), 3), dtype=torch.int32, device="cuda")
        bufs.append(d)
        outs.append(o)
        descs[i].edges, descs[i].m_directed, descs[i].n = d.data_ptr(), md, n
        descs[i].out = o.data_ptr()
    torch.cuda.synchronize()
    for budget in (0, 64 << 20):
        for o in outs:
            o.zero_()
        st = {}
        ctx.batch_dev(descs, kamsta.AlgorithmConfig(local_preprocessing=1), budget, stats=st)
        torch.cuda.synchronize()
        for i, (n, _) in enumerate(specs):
            assert descs[i].status == 0
            k = descs[i].out_count
            got = outs[i][:k].cpu().numpy().astype(np.uint32)
            alone = torch.zeros((max(n, 1), 3), dtype=torch.int32, device="cuda")
            ka = ctx.boruvka_dev(bufs[i].data_ptr(), descs[i].m_directed, n, alone.data_ptr(),
                                 kamsta.AlgorithmConfig(local_preprocessing=1, sort_output=True))
            a = alone[:ka].cpu().numpy().astype(np.uint32)
            a = a[np.lexsort((a[:, 1], a[:, 0]))]
            assert k == ka
            assert np.array_equal(got, a)
            assert descs[i].total_weight == int(a[:, 2].astype(np.uint64).sum())
        if budget:
            assert st["waves"] > 1


def test_autotune_keeps_results(kamsta):
    """kamsta_batch_autotune picks valid settings, and every setting gives the
    same forests (the tuning changes schedules, never results)."""
    import torch
    ctx = kamsta.Context(0)
    rng = np.random.default_rng(3)
    specs = [(int(2 ** rng.uniform(8, 17)), float(rng.uniform(4, 24))) for _ in range(40)]
    bufs, outs, descs = [], [], (kamsta.GraphDesc * len(specs))()
    for i, (n, deg) in enumerate(specs):
        m = min(n * (n - 1) // 2, int(n * deg / 2))
        d = torch.empty((2 * m, 3), dtype=torch.int32, device="cuda")
        md = ctx.gen_gnm_dev(n, m, 900 + i, 254, d.data_ptr())
        o = torch.zeros((max(n, 1), 3), dtype=torch.int32, device="cuda")
        bufs.append(d)
        outs.append(o)
        descs[i].edges, descs[i].m_directed, descs[i].n, descs[i].out = d.data_ptr(), md, n, \
            o.data_ptr()
    torch.cuda.synchronize()
    ref = None
    for threads, cut in [(256, 4096), (512, 32768), (1024, 16384)]:
        ctx.set_tuning(threads, cut)
        ctx.batch_dev(descs)
        torch.cuda.synchronize()
        got = [outs[i][:descs[i].out_count].cpu().numpy().copy() for i in range(len(specs))]
        if ref is None:
            ref = got
        else:
            assert all(np.array_equal(a, b) for a, b in zip(ref, got))
    t = ctx.batch_autotune(descs)
    assert t["small_threads"] in (256, 512, 1024)
    assert t["small_max_n"] in (4096, 8192, 16384, 32768)
    assert all(v > 0 for v in t["cutoff_ms"].values())
    ctx.batch_dev(descs)
    torch.cuda.synchronize()
    assert all(np.array_equal(ref[i], outs[i][:descs[i].out_count].cpu().numpy())
               for i in range(len(specs)))
