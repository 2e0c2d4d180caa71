"""The reference's binary edge files (9-byte records) streamed to the device.

The loader must produce exactly the input contract from an arbitrary record
list: (src, dst)-sorted, self loops dropped, the lightest of duplicate
entries kept, and (symmetrised) both directions present.  A numpy
restatement of that transformation is the check; the MSF of the loaded
graph is then checked against the oracle.
"""
import os

import numpy as np
import pytest

REC = np.dtype([("src", "<u4"), ("dst", "<u4"), ("w", "u1")])


def _write(path, src, dst, w):
    a = np.empty(len(src), REC)
    a["src"], a["dst"], a["w"] = src, dst, w
    a.tofile(path)


def _expected(parts, symmetrize):
    src = np.concatenate([p[0] for p in parts]).astype(np.uint64)
    dst = np.concatenate([p[1] for p in parts]).astype(np.uint64)
    w = np.concatenate([p[2] for p in parts]).astype(np.uint64)
    if symmetrize:
        src, dst, w = np.concatenate([src, dst]), np.concatenate([dst, src]), np.concatenate([w, w])
    keep = src != dst
    src, dst, w = src[keep], dst[keep], w[keep]
    order = np.lexsort((w, dst, src))
    src, dst, w = src[order], dst[order], w[order]
    first = np.ones(len(src), bool)
    first[1:] = (src[1:] != src[:-1]) | (dst[1:] != dst[:-1])
    return np.stack([src[first], dst[first], w[first]], axis=1).astype(np.uint32)


def _random_parts(rng, n, counts):
    parts = []
    for c in counts:
        s = rng.integers(0, n, c, dtype=np.uint32)
        d = rng.integers(0, n, c, dtype=np.uint32)
        d[: c // 50] = s[: c // 50]  # some self loops
        w = rng.integers(0, 256, c, dtype=np.uint8)
        k = c // 10
        if k > 0:  # duplicates with other weights
            s[c - k:] = s[:k]
            d[c - k:] = d[:k]
        parts.append((s, d, w))
    return parts


def test_capacity_and_bad_files(kamsta, tmp_path):
    """Host-only part: record counts from file sizes, size errors."""
    import ctypes as C
    p = tmp_path / "g.bin"
    _write(p, np.arange(10, dtype=np.uint32), np.arange(10, dtype=np.uint32)[::-1],
           np.ones(10, np.uint8))
    arr = (C.c_char_p * 1)(str(p).encode())
    cap = C.c_uint64()
    kamsta.check(kamsta.lib().kamsta_wedge9_capacity(arr, 1, 1, C.byref(cap)))
    assert cap.value == 20
    kamsta.check(kamsta.lib().kamsta_wedge9_capacity(arr, 1, 0, C.byref(cap)))
    assert cap.value == 10
    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"\x00" * 10)
    arr = (C.c_char_p * 1)(str(bad).encode())
    assert kamsta.lib().kamsta_wedge9_capacity(arr, 1, 1, C.byref(cap)) == kamsta._native.E_INPUT
    arr = (C.c_char_p * 1)(str(tmp_path / "missing.bin").encode())
    assert kamsta.lib().kamsta_wedge9_capacity(arr, 1, 1, C.byref(cap)) == kamsta._native.E_INPUT


@pytest.mark.gpu
@pytest.mark.parametrize("symmetrize", [True, False])
@pytest.mark.parametrize("n,counts", [(50, [200]), (1000, [3000, 1, 4000]),
                                      (1 << 16, [1 << 20, 123457])])
def test_load_matches_contract_transform(kamsta, tmp_path, symmetrize, n, counts):
    rng = np.random.default_rng(n + len(counts))
    parts = _random_parts(rng, n, counts)
    paths = []
    for i, (s, d, w) in enumerate(parts):
        p = str(tmp_path / f"part{i}.bin")
        _write(p, s, d, w)
        paths.append(p)
    ctx = kamsta.Context(0)
    edges, m, nn = ctx.load_wedge9_dev(paths, symmetrize=symmetrize)
    exp = _expected(parts, symmetrize)
    got = edges.cpu().numpy().astype(np.uint32)
    assert m == len(exp)
    assert np.array_equal(got, exp)
    allids = np.concatenate([np.concatenate([p[0], p[1]]) for p in parts])
    assert nn == int(allids.max()) + 1


@pytest.mark.gpu
def test_load_then_solve(kamsta, oracle, tmp_path):
    """GNM written as one direction per edge, unsorted: symmetrised load,
    then the MSF against Kruskal on the same (loaded) edges."""
    e = oracle.gen_gnm(1 << 14, 1 << 17, 5, 254)
    one = e[e["src"] < e["dst"]]
    perm = np.random.default_rng(1).permutation(len(one))
    p = str(tmp_path / "gnm.bin")
    _write(p, one["src"][perm], one["dst"][perm], one["w"][perm].astype(np.uint8))
    ctx = kamsta.Context(0)
    edges, m, n = ctx.load_wedge9_dev([p])
    assert m == len(e)
    host = edges.cpu().numpy().view(np.uint32).reshape(-1).view(kamsta.WEDGE)
    assert np.array_equal(host, e)  # weights <= 254 fit the 1-byte field
    import torch
    out = torch.empty((n, 3), dtype=torch.int32, device="cuda")
    k = ctx.boruvka_dev(edges.data_ptr(), m, n, out.data_ptr())
    got = out[:k].cpu().numpy().view(np.uint32).reshape(-1).view(kamsta.WEDGE)
    from tests.test_parity_gpu import _check
    _check(oracle, got, e, n)
