"""7-bit varint difference encoding (Compression::SEVEN_BIT_DIFF_ENCODING).

CPU: the library's host encoder writes, per chunk, exactly the byte stream of
the reference's encoder (varint(src - prev_src), varint(dst), varint(w);
difference_encoded_graph.hpp:175-205 with encode_value,
variable_length_encoding.hpp:6-125), restated here in Python.
GPU: the device decoder restores the edge list bit for bit, and solving from
compressed input gives the same forest as the plain entry point.
"""
import numpy as np
import pytest


def _varint(v):
    out = []
    while v >= 128:
        out.append((v & 0x7F) | 0x80)
        v >>= 7
    out.append(v)
    return out


def _py_encode_chunk(e):
    out = []
    for i in range(1, len(e)):
        out += _varint(int(e["src"][i]) - int(e["src"][i - 1]))
        out += _varint(int(e["dst"][i]))
        out += _varint(int(e["w"][i]))
    return bytes(out)


def _py_decode(cg):
    edges = []
    for c in range(cg.num_chunks):
        f = cg.first[c]
        edges.append((int(f["src"]), int(f["dst"]), int(f["w"])))
        buf = cg.data[int(cg.offset[c]):int(cg.offset[c + 1])].tobytes()
        vals, x, sh = [], 0, 0
        for b in buf:
            x |= (b & 0x7F) << sh
            sh += 7
            if not b & 0x80:
                vals.append(x)
                x, sh = 0, 0
        src = edges[-1][0]
        for k in range(0, len(vals), 3):
            src += vals[k]
            edges.append((src, vals[k + 1], vals[k + 2]))
    return edges


@pytest.mark.parametrize("chunk", [1, 3, 100, 4096])
def test_encoder_matches_reference_byte_stream(kamsta, oracle, chunk):
    e = oracle.gen_gnm(700, 3000, 4, 1 << 20)  # weights up to 2^20: multi-byte varints
    cg = kamsta.Compressed(e, 700, chunk)
    assert cg.num_chunks == (len(e) + chunk - 1) // chunk
    for c in range(cg.num_chunks):
        part = e[c * chunk:(c + 1) * chunk]
        assert cg.first[c] == part[0]
        got = cg.data[int(cg.offset[c]):int(cg.offset[c + 1])].tobytes()
        assert got == _py_encode_chunk(part)
    dec = _py_decode(cg)
    assert dec == [(int(a), int(b), int(w)) for a, b, w in zip(e["src"], e["dst"], e["w"])]


def test_encoder_size_and_errors(kamsta, oracle):
    e = oracle.gen_gnm(1 << 12, 1 << 15, 1)
    cg = kamsta.Compressed(e, 1 << 12)
    assert cg.total_bytes() < 0.7 * 12 * len(e)  # the point of the codec
    bad = e.copy()[::-1]
    with pytest.raises(kamsta.KamstaError):
        kamsta.Compressed(bad, 1 << 12)  # unsorted
    with pytest.raises(kamsta.KamstaError):
        kamsta.Compressed(e, 1 << 12, chunk_edges=5000)  # chunk too long


def _graphs(oracle):
    return [("gnm", oracle.gen_gnm(1 << 14, 1 << 17, 3), 1 << 14),
            ("gnm_wide", oracle.gen_gnm(5000, 40000, 4, 1 << 30), 5000),
            ("rgg", oracle.gen_rgg2d(1 << 15, oracle.rgg_radius(1 << 15, 12), 5), 1 << 15),
            ("rhg", oracle.gen_rhg(1 << 15, 3.0, 12, 6), 1 << 15)]


@pytest.mark.gpu
@pytest.mark.parametrize("chunk", [1, 7, 333, 2048, 4095, 4096])
def test_device_decode_roundtrip(kamsta, oracle, chunk):
    import torch
    ctx = kamsta.Context(0)
    for name, e, n in _graphs(oracle):
        cg = kamsta.Compressed(e, n, chunk)
        d = torch.zeros((len(e), 3), dtype=torch.int32, device="cuda")
        ctx.decode_7bit_dev(cg, d.data_ptr())
        torch.cuda.synchronize()
        got = d.cpu().numpy().view(np.uint32).reshape(-1).view(kamsta.WEDGE)
        assert np.array_equal(got, e), name


@pytest.mark.gpu
@pytest.mark.parametrize("chunk", [5, 2048, 4096])
def test_solve_from_compressed_equals_plain(kamsta, oracle, chunk):
    """The host container goes to the device in pieces, each decoded as it
    lands; the device container is decoded whole.  Same forest either way."""
    import torch
    ctx = kamsta.Context(0)
    from tests.test_parity_gpu import _check
    for name, e, n in _graphs(oracle):
        cg = kamsta.Compressed(e, n, chunk)
        st = {}
        got = kamsta.boruvka_7bit(cg, kamsta.AlgorithmConfig(local_preprocessing=1), stats=st)
        _check(oracle, got, e, n)
        keep, g = ctx._cgraph_dev(cg)
        out = torch.empty((n, 3), dtype=torch.int32, device="cuda")
        k = ctx.boruvka_7bit_dev(g, out.data_ptr())
        got2 = out[:k].cpu().numpy().view(np.uint32).reshape(-1).view(kamsta.WEDGE)
        _check(oracle, got2, e, n)


@pytest.mark.gpu
def test_malformed_compressed_input_is_rejected(kamsta, oracle):
    import torch
    e = oracle.gen_gnm(1000, 5000, 2)
    cg = kamsta.Compressed(e, 1000, 256)
    seg = cg.data[int(cg.offset[1]):int(cg.offset[2])]
    j = int(cg.offset[1]) + int(np.flatnonzero((seg & 0x80) == 0)[0])
    cg.data[j] |= 0x80  # the first value now runs into the next: count mismatch
    ctx = kamsta.Context(0)
    d = torch.zeros((len(e), 3), dtype=torch.int32, device="cuda")
    with pytest.raises(kamsta.KamstaError) as ei:
        ctx.decode_7bit_dev(cg, d.data_ptr())
    assert ei.value.status == kamsta._native.E_INPUT
    # the context stays usable
    ctx.decode_7bit_dev(kamsta.Compressed(e, 1000, 256), d.data_ptr())


@pytest.mark.gpu
def test_malformed_compressed_host_input_is_rejected(kamsta, oracle):
    """Through the host entry point: a value running into the next one, and
    a chunk table whose byte offsets go backwards, are input errors."""
    e = oracle.gen_gnm(1000, 5000, 2)
    cg = kamsta.Compressed(e, 1000, 256)
    seg = cg.data[int(cg.offset[1]):int(cg.offset[2])]
    j = int(cg.offset[1]) + int(np.flatnonzero((seg & 0x80) == 0)[0])
    cg.data[j] |= 0x80
    with pytest.raises(kamsta.KamstaError) as ei:
        kamsta.boruvka_7bit(cg)
    assert ei.value.status == kamsta._native.E_INPUT
    cg = kamsta.Compressed(e, 1000, 256)
    cg.offset[2], cg.offset[3] = cg.offset[3], cg.offset[2]
    with pytest.raises(kamsta.KamstaError) as ei:
        kamsta.boruvka_7bit(cg)
    assert ei.value.status == kamsta._native.E_INPUT
    # the library stays usable
    from tests.test_parity_gpu import _check
    _check(oracle, kamsta.boruvka_7bit(kamsta.Compressed(e, 1000, 256)), e, 1000)


@pytest.mark.gpu
@pytest.mark.parametrize("algo", ["boruvka", "filter_boruvka"])
def test_compression_config_on_plain_entry_points(kamsta, oracle, algo):
    """AlgorithmConfig.compression = SEVEN_BIT_DIFF_ENCODING on the plain
    entry points: the library encodes the input itself (as the reference's
    boruvka() does, hybrid_boruvka.hpp:277-299) and returns the identical
    forest as with NO_COMPRESSION, through the host and the device calls."""
    import torch
    from tests.test_parity_gpu import _check
    fn = getattr(kamsta, algo)
    ctx = kamsta.Context(0)
    for name, e, n in _graphs(oracle):
        outs = []
        for comp in (kamsta.Compression.NO_COMPRESSION,
                     kamsta.Compression.SEVEN_BIT_DIFF_ENCODING):
            cfg = kamsta.AlgorithmConfig(local_preprocessing=1, compression=comp)
            got = fn(e, cfg, n=n)
            _check(oracle, got, e, n)
            outs.append(np.sort(oracle.canon_keys(got)))
            d = torch.from_numpy(e.view(np.uint32).reshape(-1, 3).view(np.int32)).cuda()
            o = torch.empty((max(n, 1), 3), dtype=torch.int32, device="cuda")
            k = getattr(ctx, algo + "_dev")(d.data_ptr(), len(e), n, o.data_ptr(), config=cfg)
            got2 = o[:k].cpu().numpy().view(np.uint32).reshape(-1).view(kamsta.WEDGE)
            _check(oracle, got2, e, n)
        assert np.array_equal(outs[0], outs[1]), name
