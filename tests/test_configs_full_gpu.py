"""The benchmark configurations at their stated sizes, against the oracle.

* Headline configuration: GNM n = 2^26, m = 2^30 (the bench's input, seed
  2026, weights 1..254), generated on the device and solved by boruvka and
  filter_boruvka with local preprocessing; each forest must equal, edge for
  edge, the reference's own build (oracle/_ref, every vertex local) where it
  is built, else the oracle's Kruskal.
* Geometric / skewed configuration: RGG-2D and RHG (gamma 3) with n = 2^24
  vertices and average degree 16 -- the bench's exact inputs (seed 2026),
  generated on the device -- solved by filter_boruvka with and without local
  preprocessing and by boruvka; each forest must equal the oracle's Kruskal
  (base_case_mst_algos.hpp:91-112) bit for bit, and the reference's own
  build (oracle/_ref) run on the same input.
* Batched configuration: the bench's 4096 graphs (n log-uniform in [2^8,
  2^20], degree U[4, 32], GNM / RGG-2D alternating, seed 2026) in one
  kamsta_mst_batch_dev call under the 64 GB budget; every 8th graph and
  every graph with n >= 2^18 is checked against Kruskal on the host.
"""
import math
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
SEED = 2026


def _host(d, md, kamsta):
    return d[:md].cpu().numpy().view(np.uint32).reshape(-1).view(kamsta.WEDGE)


def test_headline_config_at_full_size(kamsta, oracle):
    import torch
    ctx = kamsta.Context(0)
    n, m = 1 << 26, 1 << 30
    d = torch.empty((2 * m, 3), dtype=torch.int32, device="cuda")
    md = ctx.gen_gnm_dev(n, m, SEED, 254, d.data_ptr())
    o = torch.empty((n, 3), dtype=torch.int32, device="cuda")
    cfg = kamsta.AlgorithmConfig(local_preprocessing=kamsta.LocalPreprocessing.MODIFIED_BORUVKA)
    got = {}
    for name, fn in (("boruvka", ctx.boruvka_dev), ("filter_boruvka", ctx.filter_boruvka_dev)):
        st = {}
        k = fn(d.data_ptr(), md, n, o.data_ptr(), cfg, stats=st)
        got[name] = (oracle.canon_keys(_host(o, k, kamsta)), st["total_weight"])
    e = _host(d, md, kamsta)
    del d, o
    torch.cuda.empty_cache()
    ctx.close()
    if oracle.ref_available():
        ref, rw, _ = oracle.ref_all_local(e, n)
    else:
        ref, rw = oracle.kruskal(e, n)
    want = oracle.canon_keys(ref)
    del e, ref
    for name, (keys, w) in got.items():
        assert w == rw, name
        assert np.array_equal(keys, want), name


@pytest.mark.parametrize("fam", ["rgg2d", "rhg"])
def test_geometric_config_at_full_size(kamsta, oracle, fam):
    import torch
    ctx = kamsta.Context(0)
    n = 1 << 24
    if fam == "rgg2d":
        r = math.sqrt(16.0 / (math.pi * n))
        gen = lambda **kw: ctx.gen_rgg2d_dev(n, r, SEED, 254, **kw)  # noqa: E731
    else:
        gen = lambda **kw: ctx.gen_rhg_dev(n, 3.0, 16.0, SEED, 254, **kw)  # noqa: E731
    md = gen()
    d = torch.empty((md, 3), dtype=torch.int32, device="cuda")
    gen(d_out=d.data_ptr(), capacity=md)
    torch.cuda.synchronize()
    e = _host(d, md, kamsta)
    kr, kw = oracle.kruskal(e, n)
    want = oracle.canon_keys(kr)
    LP = kamsta.LocalPreprocessing
    o = torch.empty((n, 3), dtype=torch.int32, device="cuda")
    for name, fn, lp in [("filter_boruvka", ctx.filter_boruvka_dev, LP.MODIFIED_BORUVKA),
                         ("filter_boruvka", ctx.filter_boruvka_dev, LP.NO_PREPROCESSING),
                         ("boruvka", ctx.boruvka_dev, LP.MODIFIED_BORUVKA)]:
        st = {}
        k = fn(d.data_ptr(), md, n, o.data_ptr(), kamsta.AlgorithmConfig(local_preprocessing=lp),
               stats=st)
        got = _host(o, k, kamsta)
        assert st["total_weight"] == kw, (name, lp)
        assert np.array_equal(oracle.canon_keys(got), want), (name, lp)
    if oracle.ref_available():
        ref, rw, _ = oracle.ref_all_local(e, n)
        assert rw == kw and np.array_equal(oracle.canon_keys(ref), want)
    ctx.close()


def test_batch_config_against_kruskal(kamsta, oracle):
    import torch
    from kamsta_gb300 import workloads as W
    ctx = kamsta.Context(0)
    specs = W.mixed_specs(4096, SEED)
    edges, outs, counts = W.materialize(ctx, specs)
    torch.cuda.synchronize()
    descs = W.descs_for(kamsta, specs, edges, outs, counts)
    cfg = kamsta.AlgorithmConfig(local_preprocessing=kamsta.LocalPreprocessing.MODIFIED_BORUVKA)
    ctx.batch_dev(descs, cfg, 64 << 30)
    torch.cuda.synchronize()
    check = [i for i, s in enumerate(specs) if i % 8 == 0 or s.n >= (1 << 18)]
    assert len(check) > 1000

    def one(i):
        s = specs[i]
        e = _host(edges[i], counts[i], kamsta)
        kr, kw = oracle.kruskal(e, s.n)
        k = descs[i].out_count
        got = _host(outs[i], k, kamsta)
        ok = (descs[i].status == 0 and descs[i].total_weight == kw and k == len(kr)
              and np.array_equal(oracle.canon_keys(got), oracle.canon_keys(kr)))
        return i, ok

    with ThreadPoolExecutor(4) as pool:
        bad = [i for i, ok in pool.map(one, check) if not ok]
    assert not bad, bad[:10]
    ctx.close()
