"""Serving loop: continuous batching.  Every result must be bit-identical to
the single-pair path, whether the pair runs alone or in a mix that joins the
device loop at different ticks."""
import time

import numpy as np
import pytest
import torch

from housdorffhdf5cmake_gb300 import synth

pytestmark = pytest.mark.gpu

KEYS = ("hd", "hd_ab", "hd_ba", "hd_robust", "sum_ab", "sum_ba", "n_a", "n_b", "n_a_not_b", "n_b_not_a", "status")


def same(x, y):
    return all(x[k] == y[k] for k in KEYS)


def _pairs(n, seed, lo=24, hi=96, edge=0.15):
    specs = synth.batch_ragged_specs(seed, n=n, lo=lo, hi=hi, edge_frac=edge)
    return [synth.pair_from_spec(s, "cuda") for s in specs]


def test_server_matches_plain_path(hd, ctx):
    pairs = _pairs(40, 5)
    plain = [ctx.compute(a, b, "se6") for a, b in pairs]
    with hd.Server(ctx, tick_iterations=4) as srv:
        tickets = []
        for i, (a, b) in enumerate(pairs):
            tickets.append(srv.submit(a, b))
            if i % 7 == 0:
                time.sleep(0.002)  # later arrivals join a loop already in flight
        res = [srv.wait(t, 60000) for t in tickets]
        st = srv.stats()
    for i, (r, p) in enumerate(zip(res, plain)):
        assert same(r, p), (i, r, p)
    assert st["completed"] == len(pairs) and st["ticks"] > 1


def test_alone_equals_in_mix(hd, ctx):
    pairs = _pairs(12, 9, lo=32, hi=128, edge=0.0)
    probe = pairs[3]
    with hd.Server(ctx) as srv:
        alone = srv.wait(srv.submit(*probe), 60000)
    with hd.Server(ctx, tick_iterations=2) as srv:
        ts = [srv.submit(a, b) for a, b in pairs[:3]]
        time.sleep(0.005)
        tp = srv.submit(*probe)
        ts += [srv.submit(a, b) for a, b in pairs[4:]]
        mixed = srv.wait(tp, 60000)
        for t in ts:
            srv.wait(t, 60000)
    assert same(alone, mixed)


def test_host_masks_and_se18(hd, ctx):
    pairs = _pairs(10, 11)
    host = [(a.cpu().numpy(), b.cpu().numpy()) for a, b in pairs]
    with hd.Server(ctx, metric="se18") as srv:
        ts = [srv.submit(a, b) for a, b in host]
        res = [srv.wait(t, 60000) for t in ts]
    for (a, b), r in zip(pairs, res):
        assert same(r, ctx.compute(a, b, "se18"))


def test_budget_admission_and_oversize(hd, ctx):
    pairs = _pairs(16, 13, lo=64, hi=96, edge=0.0)
    budget = 24 << 20  # a few pairs at a time
    with hd.Server(ctx, hbm_budget_bytes=budget) as srv:
        # 320^3: six 4.9 MB job buffers alone exceed the 24 MB budget
        big = torch.zeros((320, 320, 320), dtype=torch.uint8, device="cuda")
        tbig = srv.submit(big, big)
        ts = [srv.submit(a, b) for a, b in pairs]
        res = [srv.wait(t, 60000) for t in ts]
        rbig = srv.wait(tbig, 60000)
        st = srv.stats()
    assert rbig["status"] == hd.HD_ERR_OOM
    assert st["bytes_peak"] <= budget
    for (a, b), r in zip(pairs, res):
        assert same(r, ctx.compute(a, b, "se6"))


def test_cancel(hd, ctx):
    pairs = _pairs(30, 17, lo=96, hi=160, edge=0.0)
    with hd.Server(ctx, tick_iterations=1, max_inflight=4) as srv:
        ts = [srv.submit(a, b) for a, b in pairs]
        for t in ts[::3]:
            srv.cancel(t)
        res = [srv.wait(t, 60000) for t in ts]
        st = srv.stats()
    for i, ((a, b), r) in enumerate(zip(pairs, res)):
        if i % 3 == 0:
            assert r["status"] in (hd.HD_ERR_CANCELLED, hd.HD_OK)
            if r["status"] == hd.HD_OK:
                assert same(r, ctx.compute(a, b, "se6"))
        else:
            assert same(r, ctx.compute(a, b, "se6"))
    assert st["cancelled"] >= 1


@pytest.mark.parametrize("opts", [{"kernel": 1}, {"kernel": 2, "steps_per_barrier": 4}])
def test_server_kernels_and_slot_reuse(hd, ctx, opts):
    """Both dilation kernels under the server (the one-step kernel's queue
    entries and the blocked kernel's crops), with few slots so that pairs
    reuse the slots and brick ranges of finished ones."""
    pairs = _pairs(24, 23, lo=32, hi=112, edge=0.1)
    plain = [ctx.compute(a, b, "se6") for a, b in pairs]
    with hd.Context(0, **opts) as c2, hd.Server(c2, tick_iterations=3, max_inflight=3) as srv:
        ts = []
        for i, (a, b) in enumerate(pairs):
            ts.append(srv.submit(a, b))
            if i % 5 == 0:
                time.sleep(0.002)
        res = [srv.wait(t, 60000) for t in ts]
    for i, (r, p) in enumerate(zip(res, plain)):
        assert same(r, p), (opts, i, r, p)


def test_wait_any_returns_every_request(hd, ctx):
    """hd_server_wait_any hands out each finished request once, in
    completion order, with the plain path's result."""
    pairs = _pairs(20, 29, lo=32, hi=128, edge=0.1)
    plain = [ctx.compute(a, b, "se6") for a, b in pairs]
    with hd.Server(ctx) as srv:
        tickets = {srv.submit(a, b): i for i, (a, b) in enumerate(pairs)}
        got = {}
        while len(got) < len(pairs):
            t, r = srv.wait_any(60000)
            assert t in tickets and t not in got
            got[t] = r
        assert srv.wait_any(10) is None
    for t, i in tickets.items():
        assert same(got[t], plain[i]), i




def test_arrival_joins_a_running_tick(hd, ctx):
    """Continuous batching: a request submitted while a long tick runs (the
    512^3 far-blobs pair, hundreds of steps, ticks long enough to finish it
    in one) ends that tick at its next grid barrier and is admitted beside
    the big pair while the big pair still dilates (two pairs resident at
    once); both results equal the plain path."""
    big = synth.pair_far_blobs(5, (512, 512, 512), "cuda")
    small = _pairs(1, 31, lo=48, hi=64, edge=0.0)[0]
    want_big, want_small = ctx.compute(*big, "se6"), ctx.compute(*small, "se6")
    with hd.Server(ctx, tick_iterations=100000) as srv:
        tb = srv.submit(*big)
        t0 = time.time()
        while srv.stats()["resident_pairs"] == 0 and time.time() - t0 < 10:
            time.sleep(0.0002)
        time.sleep(0.001)  # the big pair's tick is running now
        ts = srv.submit(*small)
        most = 0
        while srv.stats()["completed"] == 0 and time.time() - t0 < 30:
            most = max(most, srv.stats()["resident_pairs"])
        got = dict([srv.wait_any(60000), srv.wait_any(60000)])
    assert most == 2, "the second pair was not admitted while the first one ran"
    assert same(got[ts], want_small) and same(got[tb], want_big)


def test_lone_request_then_burst_switches_kernel_shape(hd, ctx):
    """A lone request starts a busy period in the single-pair kernel shape; a
    burst submitted behind it makes the server drain and continue in the
    batch shape.  Every result equals the plain path, and a second lone
    request after the burst runs in the single-pair shape again."""
    lone = _pairs(1, 37, lo=96, hi=128, edge=0.0)[0]
    burst = _pairs(30, 41, lo=32, hi=96, edge=0.1)
    want_lone = ctx.compute(*lone, "se6")
    want = [ctx.compute(a, b, "se6") for a, b in burst]
    with hd.Server(ctx) as srv:
        t0 = srv.submit(*lone)
        time.sleep(0.0005)
        ts = [srv.submit(a, b) for a, b in burst]
        res = [srv.wait(t, 60000) for t in ts]
        r0 = srv.wait(t0, 60000)
        time.sleep(0.002)
        r1 = srv.wait(srv.submit(*lone), 60000)
    assert same(r0, want_lone) and same(r1, want_lone)
    for i, (r, w) in enumerate(zip(res, want)):
        assert same(r, w), i
