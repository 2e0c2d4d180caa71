"""Serving loop (kamsta_server_*): every job's forest is the same when it is
solved alone and when it is solved in a mix of concurrently submitted jobs
spread over several waves and workers (exact: byte-identical output, equal
to the plain solver's forest sorted by (src, dst))."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _graphs(kamsta, ctx, count, seed):
    import torch
    rng = np.random.default_rng(seed)
    gs = []
    for i in range(count):
        n = int(2 ** rng.uniform(8, 14))
        deg = float(rng.uniform(4, 32))
        if i % 2 == 0:
            m = min(n * (n - 1) // 2, int(n * deg / 2))
            d = torch.empty((max(2 * m, 1), 3), dtype=torch.int32, device="cuda")
            md = ctx.gen_gnm_dev(n, m, 1000 * seed + i, 254, d.data_ptr())
        else:
            r = (deg / (np.pi * n)) ** 0.5
            md = ctx.gen_rgg2d_dev(n, r, 1000 * seed + i, 254)
            d = torch.empty((max(md, 1), 3), dtype=torch.int32, device="cuda")
            ctx.gen_rgg2d_dev(n, r, 1000 * seed + i, 254, d.data_ptr(), md)
        gs.append((d, md, n))
    torch.cuda.synchronize()
    return gs


def _drain(server, want, timeout_s=120):
    got = {}
    t0 = time.time()
    while len(got) < want:
        for c in server.poll(timeout_us=100000):
            got[c["tag"]] = c
        assert time.time() - t0 < timeout_s, "server did not finish"
    return got


def _plain(kamsta, ctx, d, md, n):
    import torch
    o = torch.zeros((max(n, 1), 3), dtype=torch.int32, device="cuda")
    k = ctx.boruvka_dev(d.data_ptr(), md, n, o.data_ptr())
    a = o[:k].cpu().numpy().astype(np.uint32)
    return a[np.lexsort((a[:, 1], a[:, 0]))]


def test_same_result_alone_and_in_mix(kamsta):
    import torch
    ctx = kamsta.Context(0)
    gs = _graphs(kamsta, ctx, 40, 3)
    outs_alone = [torch.zeros((max(n, 1), 3), dtype=torch.int32, device="cuda")
                  for _, _, n in gs]
    outs_mix = [torch.zeros((max(n, 1), 3), dtype=torch.int32, device="cuda") for _, _, n in gs]
    # alone: one job at a time
    srv = kamsta.Server(0, workers=1)
    alone = {}
    for i, (d, md, n) in enumerate(gs):
        srv.submit(d.data_ptr(), md, n, outs_alone[i].data_ptr(), tag=i)
        c = _drain(srv, 1)
        assert c[i]["batch_size"] == 1
        alone[i] = c[i]
    srv.close()
    # in the mix: all at once, 3 workers, a budget that forces several waves
    srv = kamsta.Server(0, budget_bytes=3 * (48 << 20), workers=3)
    for i, (d, md, n) in enumerate(gs):
        srv.submit(d.data_ptr(), md, n, outs_mix[i].data_ptr(), tag=i)
    mix = _drain(srv, len(gs))
    waves = srv.stats()["waves"]
    mem = srv.memory()
    srv.close()
    assert waves > 1
    # the budget is enforced: no worker's context went over its share
    assert mem["worker_limit"] == 48 << 20
    assert 0 < mem["peak_worker_bytes"] <= mem["worker_limit"]
    assert max(c["batch_size"] for c in mix.values()) > 1
    for i, (d, md, n) in enumerate(gs):
        assert alone[i]["status"] == 0 and mix[i]["status"] == 0
        k = alone[i]["out_count"]
        assert mix[i]["out_count"] == k
        assert mix[i]["total_weight"] == alone[i]["total_weight"]
        a = outs_alone[i][:k].cpu().numpy().astype(np.uint32)
        b = outs_mix[i][:k].cpu().numpy().astype(np.uint32)
        assert np.array_equal(a, b)
        assert np.array_equal(a, _plain(kamsta, ctx, d, md, n))
        assert alone[i]["submit_us"] <= alone[i]["start_us"] <= alone[i]["finish_us"]


def test_budget_rejects_oversized_job(kamsta):
    import torch
    ctx = kamsta.Context(0)
    (d, md, n), = _graphs(kamsta, ctx, 1, 9)
    out = torch.zeros((n, 3), dtype=torch.int32, device="cuda")
    srv = kamsta.Server(0, budget_bytes=1 << 16, workers=1)
    with pytest.raises(kamsta.KamstaError) as ei:
        srv.submit(d.data_ptr(), md, n, out.data_ptr())
    assert ei.value.status == kamsta._native.E_BUDGET
    srv.close()


def test_bad_job_does_not_disturb_mix(kamsta):
    import torch
    ctx = kamsta.Context(0)
    gs = _graphs(kamsta, ctx, 8, 5)
    d, md, n = gs[3]
    bad = d.clone()
    bad[md // 2, 1] = n + 5  # a dst id >= n
    gs[3] = (bad, md, n)
    outs = [torch.zeros((max(n, 1), 3), dtype=torch.int32, device="cuda") for _, _, n in gs]
    srv = kamsta.Server(0, workers=2)
    for i, (d, md, n) in enumerate(gs):
        srv.submit(d.data_ptr(), md, n, outs[i].data_ptr(), tag=i)
    got = _drain(srv, len(gs))
    srv.close()
    for i, (d, md, n) in enumerate(gs):
        if i == 3:
            assert got[i]["status"] == kamsta._native.E_INPUT
            continue
        assert got[i]["status"] == 0
        k = got[i]["out_count"]
        assert np.array_equal(outs[i][:k].cpu().numpy().astype(np.uint32),
                              _plain(kamsta, ctx, d, md, n))


def test_cancel_queued_job(kamsta):
    import torch
    ctx = kamsta.Context(0)
    # a large job keeps the single worker busy while the others queue
    nb, mb = 1 << 21, 1 << 25
    big = torch.empty((2 * mb, 3), dtype=torch.int32, device="cuda")
    assert ctx.gen_gnm_dev(nb, mb, 77, 254, big.data_ptr()) == 2 * mb
    out_big = torch.zeros((nb, 3), dtype=torch.int32, device="cuda")
    gs = _graphs(kamsta, ctx, 6, 11)
    outs = [torch.zeros((max(n, 1), 3), dtype=torch.int32, device="cuda") for _, _, n in gs]
    srv = kamsta.Server(0, workers=1)
    t_big = srv.submit(big.data_ptr(), 2 * mb, nb, out_big.data_ptr(), tag=100)
    t0 = time.time()
    while srv.stats()["in_flight"] == 0:
        assert time.time() - t0 < 30, "the worker did not take the large job"
        time.sleep(0.0002)
    tickets = [srv.submit(d.data_ptr(), md, n, outs[i].data_ptr(), tag=i)
               for i, (d, md, n) in enumerate(gs)]
    assert srv.cancel(tickets[2])
    assert not srv.cancel(tickets[2])        # no longer queued
    assert not srv.cancel(t_big)             # already in a wave
    assert not srv.cancel(10 ** 12)          # unknown ticket
    got = _drain(srv, len(gs) + 1)
    srv.close()
    assert got[2]["status"] == kamsta._native.E_CANCELLED
    assert got[2]["batch_size"] == 0 and got[2]["out_count"] == 0
    assert not outs[2].any()                 # its buffers were never touched
    assert got[100]["status"] == 0
    k = got[100]["out_count"]
    assert np.array_equal(out_big[:k].cpu().numpy().astype(np.uint32),
                          _plain(kamsta, ctx, big, 2 * mb, nb))
    for i, (d, md, n) in enumerate(gs):
        if i == 2:
            continue
        assert got[i]["status"] == 0
        k = got[i]["out_count"]
        assert np.array_equal(outs[i][:k].cpu().numpy().astype(np.uint32),
                              _plain(kamsta, ctx, d, md, n))


def test_job_submitted_mid_wave_overlaps_and_finishes_first(kamsta):
    """Continuous batching: while worker 0 solves a large job, a small job
    submitted after that wave started is taken by the other worker, its
    [start, finish] interval overlaps the large job's, and it finishes
    first; both forests equal the plain solver's."""
    import torch
    ctx = kamsta.Context(0)
    nb, mb = 1 << 24, 1 << 28                 # about 25 ms of device work
    big = torch.empty((2 * mb, 3), dtype=torch.int32, device="cuda")
    assert ctx.gen_gnm_dev(nb, mb, 78, 254, big.data_ptr()) == 2 * mb
    out_big = torch.zeros((nb, 3), dtype=torch.int32, device="cuda")
    (d, md, n), = _graphs(kamsta, ctx, 1, 12)
    out = torch.zeros((max(n, 1), 3), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    srv = kamsta.Server(0, budget_bytes=2 * (40 << 30), workers=2)
    srv.submit(big.data_ptr(), 2 * mb, nb, out_big.data_ptr(), tag=1)
    t0 = time.time()
    while srv.stats()["in_flight"] == 0:
        assert time.time() - t0 < 30, "no worker took the large job"
        time.sleep(0.0001)
    srv.submit(d.data_ptr(), md, n, out.data_ptr(), tag=2)
    got = _drain(srv, 2)
    mem = srv.memory()
    srv.close()
    a, b = got[1], got[2]
    assert a["status"] == 0 and b["status"] == 0
    assert a["batch_size"] == 1 and b["batch_size"] == 1    # two separate waves
    # submitted after the large job's wave was taken (in_flight > 0); its
    # start stamp is taken a few microseconds after that, so compare submits
    assert b["submit_us"] > a["submit_us"]
    assert b["start_us"] < a["finish_us"]                  # the intervals overlap
    assert b["finish_us"] < a["finish_us"]                 # and it finished first
    assert mem["peak_worker_bytes"] <= mem["worker_limit"]
    k = b["out_count"]
    assert np.array_equal(out[:k].cpu().numpy().astype(np.uint32), _plain(kamsta, ctx, d, md, n))
    k = a["out_count"]
    assert np.array_equal(out_big[:k].cpu().numpy().astype(np.uint32),
                          _plain(kamsta, ctx, big, 2 * mb, nb))


def test_worker_share_is_the_job_limit(kamsta):
    """A job that fits the whole budget but not one worker's share is refused
    (each worker's context is limited to budget / workers)."""
    import torch
    ctx = kamsta.Context(0)
    (d, md, n), = _graphs(kamsta, ctx, 1, 13)
    out = torch.zeros((max(n, 1), 3), dtype=torch.int32, device="cuda")
    srv = kamsta.Server(0, budget_bytes=8 << 20, workers=4)    # 2 MiB per worker
    with pytest.raises(kamsta.KamstaError) as ei:
        srv.submit(d.data_ptr(), md, n, out.data_ptr())
    assert ei.value.status == kamsta._native.E_BUDGET
    srv.close()
