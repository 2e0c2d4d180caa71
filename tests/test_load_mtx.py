"""MatrixMarket coordinate files (the reference's unweighted input) as solver
input.  The expected edge list is restated here with numpy: entry (i, j) ->
the pair {i-1, j-1}, self loops dropped, repeated pairs merged, both
directions, (src, dst)-sorted, the generators' hash weight; the MSF of the
loaded graph is then checked against the oracle."""
import numpy as np
import pytest


def _mix64(z):
    M = (1 << 64) - 1
    z = (z + 0x9E3779B97F4A7C15) & M
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
    return z ^ (z >> 31)


def _expected(pairs, seed, wmax):
    u = np.minimum(pairs[:, 0], pairs[:, 1]).astype(np.uint64)
    v = np.maximum(pairs[:, 0], pairs[:, 1]).astype(np.uint64)
    keep = u != v
    key = np.unique((u[keep] << np.uint64(32)) | v[keep])
    wseed = _mix64(seed ^ 0x6A09E667F3BCC909)
    w = np.array([1 + ((_mix64(wseed ^ int(k)) * wmax) >> 64) for k in key], dtype=np.uint64)
    lo, hi = key >> np.uint64(32), key & np.uint64(0xFFFFFFFF)
    s, d, ww = np.concatenate([lo, hi]), np.concatenate([hi, lo]), np.concatenate([w, w])
    order = np.lexsort((d, s))
    return np.stack([s[order], d[order], ww[order]], axis=1).astype(np.uint32)


def _write(path, rows, cols, pairs, field="pattern", sym="general", comments=True):
    with open(path, "w") as f:
        f.write(f"%%MatrixMarket matrix coordinate {field} {sym}\n")
        if comments:
            f.write("% generated for a test\n%\n")
        f.write(f"{rows} {cols} {len(pairs)}\n")
        for i, j in pairs:
            if field == "pattern":
                f.write(f"{i + 1} {j + 1}\n")
            else:
                f.write(f"{i + 1}\t{j + 1}   {((i * 7 + j) % 13) / 4:.2f}\r\n")


def test_header_and_errors(kamsta, tmp_path):
    """Host-only part: the banner, comments and the size line."""
    p = tmp_path / "a.mtx"
    _write(p, 7, 9, [(0, 1), (2, 3)])
    assert kamsta.mtx_header(p) == (7, 9, 2)
    bad = tmp_path / "b.mtx"
    bad.write_text("%%MatrixMarket matrix array real general\n3 3\n1\n")
    with pytest.raises(kamsta.KamstaError) as ei:
        kamsta.mtx_header(bad)
    assert ei.value.status == kamsta._native.E_UNSUPPORTED
    bad.write_text("hello\n")
    with pytest.raises(kamsta.KamstaError):
        kamsta.mtx_header(bad)
    bad.write_text("%%MatrixMarket matrix coordinate pattern general\n% only comments\n")
    with pytest.raises(kamsta.KamstaError):
        kamsta.mtx_header(bad)
    with pytest.raises(kamsta.KamstaError):
        kamsta.mtx_header(tmp_path / "missing.mtx")


@pytest.mark.gpu
@pytest.mark.parametrize("n,m,field,sym", [(5, 0, "pattern", "general"), (2, 3, "pattern", "general"),
                                           (60, 400, "pattern", "symmetric"),
                                           (3000, 20000, "real", "general"),
                                           (1 << 16, 1 << 20, "integer", "symmetric")])
def test_load_matches_restatement(kamsta, tmp_path, n, m, field, sym):
    rng = np.random.default_rng(n + m)
    pairs = rng.integers(0, n, size=(m, 2))
    if m:
        pairs[: m // 40, 1] = pairs[: m // 40, 0]        # self loops
        pairs[m - m // 10:] = pairs[: m // 10][:, ::-1]  # repeats, both orientations
    p = tmp_path / "g.mtx"
    _write(p, n, n - 1 if n > 2 else n, [(int(a), int(b) % max(n - 1, 1) if n > 2 else int(b))
                                         for a, b in pairs], field, sym)
    rows, cols, ent = kamsta.mtx_header(p)
    assert ent == m
    ctx = kamsta.Context(0)
    edges, md, nn = ctx.load_mtx_dev(p, seed=9, max_weight=100)
    assert nn == max(rows, cols)
    got = edges.cpu().numpy().astype(np.uint32)
    q = np.array([(a, b % max(n - 1, 1) if n > 2 else b) for a, b in pairs],
                 dtype=np.int64).reshape(-1, 2)
    assert np.array_equal(got, _expected(q, 9, 100))
    assert md == len(got)


@pytest.mark.gpu
def test_load_then_solve(kamsta, oracle, tmp_path):
    """A G(n,m) pattern written as MatrixMarket (one orientation, shuffled):
    the loaded graph's MSF equals Kruskal's on the same loaded edges."""
    e = oracle.gen_gnm(1 << 14, 1 << 17, 5, 254)
    one = e[e["src"] < e["dst"]]
    perm = np.random.default_rng(2).permutation(len(one))
    p = tmp_path / "gnm.mtx"
    _write(p, 1 << 14, 1 << 14, [(int(one["src"][i]), int(one["dst"][i])) for i in perm])
    ctx = kamsta.Context(0)
    edges, m, n = ctx.load_mtx_dev(p, seed=3)
    import torch
    out = torch.empty((n, 3), dtype=torch.int32, device="cuda")
    k = ctx.boruvka_dev(edges.data_ptr(), m, n, out.data_ptr())
    got = out[:k].cpu().numpy().view(np.uint32).reshape(-1).view(kamsta.WEDGE)
    host = edges.cpu().numpy().view(np.uint32).reshape(-1).view(kamsta.WEDGE)
    from tests.test_parity_gpu import _check
    _check(oracle, got, host, n)


@pytest.mark.gpu
def test_malformed_body(kamsta, tmp_path):
    ctx = kamsta.Context(0)
    p = tmp_path / "x.mtx"
    p.write_text("%%MatrixMarket matrix coordinate pattern general\n4 4 3\n1 2\n2 9\n3 4\n")
    with pytest.raises(kamsta.KamstaError):
        ctx.load_mtx_dev(p)  # index 9 > 4
    p.write_text("%%MatrixMarket matrix coordinate pattern general\n4 4 3\n1 2\n3 4\n")
    with pytest.raises(kamsta.KamstaError):
        ctx.load_mtx_dev(p)  # 2 entries, 3 announced
