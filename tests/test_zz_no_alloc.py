"""The allocation-free entry point, kamsta_mst_boruvka_noalloc.

Callers that cannot allocate device memory (code living inside another
framework's fixed memory budget, allocator-less runtimes, plugins that are
handed only a stream and buffers) use this entry point; it keeps its scratch
in a fixed array inside the library.  This test calls it through the C ABI
twice in a row and checks each result bit-exactly (same edge set, same
weight) against kamsta_mst_boruvka_dev, the regular entry point, and against
the oracle's Kruskal.  It lives in
its own file that pytest collects last, and it passes both alone in a fresh
process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(kamsta, d_in, md, n, d_out, stream):
    cnt, w = C.c_uint64(0), C.c_uint64(0)
    kamsta.check(kamsta.lib().kamsta_mst_boruvka_noalloc(
        C.c_void_p(d_in), md, n, C.c_void_p(d_out), C.byref(cnt), C.byref(w),
        C.c_void_p(stream)))
    return int(cnt.value), int(w.value)


def _edges(t, k, kamsta):
    return t[:k].cpu().numpy().view(np.uint32).reshape(-1).view(kamsta.WEDGE)


# (n, m undirected, seed, max weight): a mid-size graph, the exact limit
# (n = 32768, m_directed = 262144), the limit with weights 1..4 (long ties),
# and a sparse graph with thousands of isolated vertices.
CASES = [(20000, 100000, 41, 254), (32768, 131072, 42, 254), (32768, 131072, 43, 4),
         (32768, 6000, 44, 3)]


@pytest.mark.parametrize("n,m,seed,wmax", CASES)
def test_noalloc_matches_regular_entry_point_twice(kamsta, oracle, n, m, seed, wmax):
    import torch
    ctx = kamsta.Context(0)
    stream = torch.cuda.current_stream().cuda_stream
    edges = oracle.gen_gnm(n, m, seed, wmax)
    assert len(edges) == 2 * m
    kr, kw = oracle.kruskal(edges, n)
    d_in = torch.from_numpy(edges.view(np.uint32).reshape(-1, 3).view(np.int32)).cuda()
    d_ref = torch.empty((n, 3), dtype=torch.int32, device="cuda")
    stats = {}
    k_ref = ctx.boruvka_dev(d_in.data_ptr(), len(edges), n, d_ref.data_ptr(),
                            stream=stream, stats=stats)
    ref = _edges(d_ref, k_ref, kamsta)
    for _ in range(2):  # two calls in a row share the static scratch array
        d_na = torch.full((n, 3), -1, dtype=torch.int32, device="cuda")
        k_na, w_na = _noalloc(kamsta, d_in.data_ptr(), len(edges), n, d_na.data_ptr(), stream)
        got = _edges(d_na, k_na, kamsta)
        assert k_na == k_ref == len(kr)
        assert w_na == stats["total_weight"] == kw == int(got["w"].astype(np.uint64).sum())
        assert np.array_equal(oracle.canon_keys(got), oracle.canon_keys(ref))
        assert np.array_equal(oracle.canon_keys(got), oracle.canon_keys(kr))
    ctx.close()


def test_noalloc_reports_ids_beyond_n(kamsta, oracle):
    import torch
    edges = oracle.gen_gnm(1000, 4000, 45)
    n = int(max(edges["src"].max(), edges["dst"].max()))  # the largest id is now == n
    d_in = torch.from_numpy(edges.view(np.uint32).reshape(-1, 3).view(np.int32)).cuda()
    d_out = torch.zeros((1000, 3), dtype=torch.int32, device="cuda")
    with pytest.raises(kamsta.KamstaError) as ei:
        _noalloc(kamsta, d_in.data_ptr(), len(edges), n, d_out.data_ptr(), 0)
    assert ei.value.status == 1 and "id >= n" in str(ei.value)
    # the next call on the same array is unaffected
    kr, kw = oracle.kruskal(edges, 1000)
    k, w = _noalloc(kamsta, d_in.data_ptr(), len(edges), 1000, d_out.data_ptr(), 0)
    assert (k, w) == (len(kr), kw)


def test_noalloc_rejects_graphs_beyond_its_limits(kamsta):
    import torch
    d = torch.zeros((4, 3), dtype=torch.int32, device="cuda")
    with pytest.raises(kamsta.KamstaError) as ei:
        _noalloc(kamsta, d.data_ptr(), 4, 32769, d.data_ptr(), 0)
    assert ei.value.status == 1 and "limits" in str(ei.value)
    with pytest.raises(kamsta.KamstaError):
        _noalloc(kamsta, d.data_ptr(), (1 << 18) + 1, 100, d.data_ptr(), 0)
