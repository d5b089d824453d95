"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

Integer results must be bit-identical: hd, one-sided HDs, the exact distance
sums and the voxel counts; avg_hd is the same double division of the same
integers.  The oracle restates forBench/HausdorffDistance.cu:101-187 and is
itself pinned against breadth-first search and brute force (test_oracle.py).
"""
import math

import numpy as np
import pytest
import torch

from housdorffhdf5cmake_gb300 import synth

pytestmark = pytest.mark.gpu

KEYS = ("hd", "hd_ab", "hd_ba", "sum_ab", "sum_ba", "n_a", "n_b", "n_a_not_b", "n_b_not_a", "status")


def assert_same(g, o, what=""):
    for k in KEYS:
        assert g[k] == o[k], f"{what} {k}: gpu {g[k]} oracle {o[k]}\n gpu={g}\n oracle={o}"
    if o["status"] == 0:
        assert g["avg_hd"] == o["avg_hd"], what
    elif o["status"] == 1:
        assert math.isnan(g["avg_hd"]), what


def cuda(x):
    if isinstance(x, np.ndarray):
        x = torch.from_numpy(x)
    return x.to("cuda")


def random_pair(rng, shape, p_a=0.01, p_b=0.01, blobs=True):
    D, H, W = shape
    a = (rng.random(shape) < p_a).astype(np.uint8)
    b = (rng.random(shape) < p_b).astype(np.uint8)
    if blobs and min(shape) >= 4:
        ta, tb = torch.from_numpy(a), torch.from_numpy(b)
        for t in (ta, tb):
            c = [int(rng.integers(0, n)) for n in (W, H, D)]
            r = [int(rng.integers(1, max(2, n // 3))) for n in (W, H, D)]
            synth.draw_ellipsoid_into(t, c, r)
        a, b = ta.numpy(), tb.numpy()
    return a, b


@pytest.mark.parametrize("metric", ["se6", "se18"])
@pytest.mark.parametrize("seed", [1, 2, 3, 4, 5, 6])
def test_ellipsoid_salt_64(ctx, oracle, metric, seed):
    a, b = synth.pair_ellipsoid_salt(seed)
    a, b = a.numpy(), b.numpy()
    o = oracle.forbench(a, b, metric)
    g = ctx.compute(cuda(a), cuda(b), metric)
    assert_same(g, o, f"seed {seed}")
    if metric == "se6":
        bf = oracle.bruteforce_l1(a, b)
        assert_same(g, bf, f"brute seed {seed}")


SHAPES = [
    (1, 1, 1), (1, 1, 2), (1, 37, 1), (70, 1, 1), (1, 1, 70), (1, 40, 50), (5, 3, 33), (7, 64, 65),
    (3, 17, 129), (33, 31, 95), (9, 2, 31), (2, 9, 32), (17, 23, 64), (16, 16, 160), (4, 100, 7),
]


@pytest.mark.parametrize("metric", ["se6", "se18"])
@pytest.mark.parametrize("shape", SHAPES)
def test_ragged_shapes(ctx, oracle, metric, shape):
    rng = np.random.default_rng(hash(shape) % (2**32))
    for trial in range(3):
        a, b = random_pair(rng, shape, p_a=0.02 * (trial + 1), p_b=0.01, blobs=trial > 0)
        o = oracle.forbench(a, b, metric)
        g = ctx.compute(cuda(a), cuda(b), metric)
        assert_same(g, o, f"{shape} trial {trial}")


@pytest.mark.parametrize("metric", ["se6", "se18"])
def test_edge_cases(ctx, oracle, metric):
    shape = (20, 30, 70)
    z = np.zeros(shape, np.uint8)
    one = z.copy()
    one[3, 4, 5] = 1
    far = z.copy()
    far[-1, -1, -1] = 1
    full = np.ones(shape, np.uint8)
    border = z.copy()
    border[0, :, :] = 1
    border[:, :, -1] = 1
    cases = {
        "both_empty": (z, z),
        "a_empty": (z, one),
        "b_empty": (one, z),
        "identical": (one, one.copy()),
        "corners": (one, far),
        "corner_to_corner": (far, np.flip(far).copy()),
        "full_vs_point": (full, one),
        "border_planes": (border, far),
        "full_vs_full": (full, full.copy()),
    }
    for name, (a, b) in cases.items():
        o = oracle.forbench(a, b, metric)
        g = ctx.compute(cuda(a), cuda(b), metric)
        assert_same(g, o, name)


@pytest.mark.parametrize("metric", ["se6", "se18"])
def test_brick_shapes_agree(hd, oracle, metric):
    a, b = synth.pair_shifted_union(11, (48, 96, 160), "cpu", rmin=5, rmax=30, max_shift=8)
    a, b = a.numpy(), b.numpy()
    o = oracle.bfs_pair(a, b, metric)
    da, db = cuda(a), cuda(b)
    for bxw in (2, 4, 8):
        for bz in (4, 8, 16):
            for cps in (0, 1):
                with hd.Context(0, kernel=1, brick_x_words=bxw, brick_z=bz, ctas_per_sm=cps) as c:
                    g = c.compute(da, db, metric)
                assert_same(g, o, f"one-step kernel brick {bxw}x{bz} cps {cps}")
    for steps, bz in ((1, 8), (1, 16), (2, 8), (2, 16), (3, 8), (4, 8), (5, 8)):
        for cps in (0, 1):
            with hd.Context(0, kernel=2, steps_per_barrier=steps, brick_z=bz, ctas_per_sm=cps) as c:
                g = c.compute(da, db, metric)
            assert_same(g, o, f"blocked kernel {steps} steps bz {bz} cps {cps}")


@pytest.mark.parametrize("metric", ["se6", "se18"])
@pytest.mark.parametrize("kernel,steps", [(1, 0), (2, 1), (2, 2), (2, 3), (2, 4), (2, 5)])
def test_kernels_on_ragged_shapes(hd, oracle, metric, kernel, steps):
    rng = np.random.default_rng(7)
    with hd.Context(0, kernel=kernel, steps_per_barrier=steps) as c:
        for shape in SHAPES:
            a, b = random_pair(rng, shape, p_a=0.03, p_b=0.01)
            assert_same(c.compute(cuda(a), cuda(b), metric), oracle.forbench(a, b, metric), f"{shape}")


def test_shifted_union_midsize(ctx, oracle):
    for seed in (21, 22):
        a, b = synth.pair_shifted_union(seed, (96, 160, 192), "cpu", rmin=8, rmax=40, max_shift=12)
        a, b = a.numpy(), b.numpy()
        for metric in ("se6", "se18"):
            o = oracle.bfs_pair(a, b, metric)
            g = ctx.compute(cuda(a), cuda(b), metric)
            assert_same(g, o, f"seed {seed} {metric}")


def test_host_device_and_zero_copy_paths(hd, ctx, oracle):
    a, b = synth.pair_shifted_union(5, (40, 72, 100), "cpu", rmin=5, rmax=20, max_shift=6)
    an, bn = a.numpy(), b.numpy()
    o = oracle.bfs_pair(an, bn, "se6")
    assert_same(ctx.compute(an, bn, "se6"), o, "pageable host")
    assert_same(ctx.compute(a.pin_memory(), b.pin_memory(), "se6"), o, "pinned host")
    assert_same(ctx.compute(cuda(an), cuda(bn), "se6"), o, "device")
    with hd.Context(0, zero_copy=False) as c:
        assert_same(c.compute(an, bn, "se6"), o, "staged copy")
    # unaligned device pointers take the byte-load packing path
    big_a = torch.zeros(an.size + 3, dtype=torch.uint8, device="cuda")
    big_b = torch.zeros(an.size + 5, dtype=torch.uint8, device="cuda")
    va = big_a[3:].view(an.shape)
    vb = big_b[5:].view(an.shape)
    va.copy_(cuda(an))
    vb.copy_(cuda(bn))
    assert va.data_ptr() % 16 != 0
    assert_same(ctx.compute(va, vb, "se6"), o, "unaligned device")


# x extents (first, last word) of A u B: the blocked kernel reads the packed
# masks in place when its domain can start on a multiple of 4 words without
# an extra brick column (e.g. words 2-3, 4-6), else crops of A and B (words
# 1-4, 3-4); batches always read in place.
WORD_EXTENTS = [(0, 0), (1, 4), (2, 3), (3, 3), (3, 4), (4, 6), (5, 7), (1, 7), (6, 6)]


def _pair_in_words(rng, shape, w0, w1):
    D, H, W = shape
    x0, x1 = 32 * w0, min(W, 32 * (w1 + 1)) - 1
    a = np.zeros(shape, np.uint8)
    b = np.zeros(shape, np.uint8)
    for m, p in ((a, 0.03), (b, 0.02)):
        m[:, :, x0:x1 + 1] = rng.random((D, H, x1 - x0 + 1)) < p
    a[D // 2, H // 3, x0] = 1  # both ends of the extent
    b[D // 3, H // 2, x1] = 1
    return a, b


@pytest.mark.parametrize("metric", ["se6", "se18"])
@pytest.mark.parametrize("width", [256, 200])
def test_blocked_domain_origins(hd, oracle, metric, width):
    rng = np.random.default_rng(width)
    shape = (12, 40, width)
    pairs = [_pair_in_words(rng, shape, w0, w1) for w0, w1 in WORD_EXTENTS if 32 * w0 < width]
    want = [oracle.forbench(a, b, metric) for a, b in pairs]
    for steps in (1, 4):
        with hd.Context(0, kernel=2, steps_per_barrier=steps) as c:
            for (a, b), o, ext in zip(pairs, want, WORD_EXTENTS):
                assert_same(c.compute(cuda(a), cuda(b), metric), o, f"words {ext} steps {steps}")
            got = c.batch([(cuda(a), cuda(b)) for a, b in pairs], metric)
            for g, o, ext in zip(got, want, WORD_EXTENTS):
                assert_same(g, o, f"batch words {ext} steps {steps}")


def test_batch_equals_plain(ctx, oracle):
    specs = synth.batch_ragged_specs(3, n=24, lo=16, hi=80, edge_frac=0.2)
    pairs = [synth.pair_from_spec(s) for s in specs]
    for metric in ("se6", "se18"):
        dev = [(cuda(a), cuda(b)) for a, b in pairs]
        batch = ctx.batch(dev, metric)
        for i, ((a, b), g) in enumerate(zip(pairs, batch)):
            plain = ctx.compute(dev[i][0], dev[i][1], metric)
            assert_same(g, plain, f"pair {i} batch vs plain")
            o = oracle.forbench(a.numpy(), b.numpy(), metric)
            assert_same(g, o, f"pair {i} vs oracle ({specs[i].kind})")
        # host masks in a batch
        host = ctx.batch([(a.numpy(), b.numpy()) for a, b in pairs[:6]], metric)
        for i in range(6):
            assert_same(host[i], batch[i], f"host batch pair {i}")


def test_robust_hd(hd, oracle):
    a, b = synth.pair_shifted_union(8, (40, 80, 96), "cpu", rmin=5, rmax=25, max_shift=10)
    a, b = a.numpy(), b.numpy()
    o = oracle.forbench(a, b, "se6", hist=True)
    for p in (0.5, 0.9, 0.95, 1.0):
        with hd.Context(0, percentile=p) as c:
            g = c.compute(cuda(a), cuda(b), "se6")
        want = oracle.robust_hd(o["hist_ab"], o["hist_ba"], o["n_a_not_b"], o["n_b_not_a"], p)
        assert g["hd_robust"] == want, p
    assert g["hd_robust"] == o["hd"]


@pytest.mark.parametrize("metric", ["se6", "se18"])
def test_profile_tile_counts(ctx, oracle, metric):
    a, b = synth.pair_shifted_union(9, (70, 90, 130), "cpu", rmin=6, rmax=30, max_shift=10)
    a, b = a.numpy(), b.numpy()
    g, tab, tba, bricks = ctx.profile(cuda(a), cuda(b), metric)
    o = oracle.bfs_pair(a, b, metric)
    assert_same(g, o)
    D, H, W = a.shape
    # the domain: the bounding box of A u B, x in whole words; the
    # 18-neighbour element widens it by a word, a row and a plane
    zz, yy, xx = np.nonzero(a | b)
    m = 0 if metric == "se6" else 1
    w0, w1 = max(0, xx.min() // 32 - m), min((W - 1) // 32, xx.max() // 32 + m)
    box = (32 * w0, min(W - 1, 32 * w1 + 31), max(0, yy.min() - m), min(H - 1, yy.max() + m),
           max(0, zz.min() - m), min(D - 1, zz.max() + m))
    da = oracle.bfs_dt(a, metric)
    db = oracle.bfs_dt(b, metric)
    want_ba = oracle.tile_counts(da, box, g["hd_ba"])
    want_ab = oracle.tile_counts(db, box, g["hd_ab"])
    assert list(tba[: g["hd_ba"] + 1]) == list(want_ba)
    assert list(tab[: g["hd_ab"] + 1]) == list(want_ab)
    assert bricks > 0


@pytest.mark.parametrize("metric", ["se6", "se18"])
def test_distance_maps(ctx, oracle, metric):
    a, b = synth.pair_shifted_union(12, (30, 64, 80), "cpu", rmin=4, rmax=18, max_shift=7)
    a, b = a.numpy(), b.numpy()
    g, ma, mb = ctx.distance_map(cuda(a), cuda(b), metric)
    da = oracle.bfs_dt(a, metric)
    db = oracle.bfs_dt(b, metric)
    want_a = np.where(a != 0, np.where(b != 0, 0, db), -1)
    want_b = np.where(b != 0, np.where(a != 0, 0, da), -1)
    np.testing.assert_array_equal(ma.cpu().numpy(), want_a)
    np.testing.assert_array_equal(mb.cpu().numpy(), want_b)
    assert int(ma.max()) == g["hd_ab"] and int(mb.max()) == g["hd_ba"]


def test_determinism(ctx):
    a, b = synth.pair_shifted_union(4, (64, 128, 128), "cuda", rmin=8, rmax=40, max_shift=12)
    first = ctx.compute(a, b, "se6")
    for _ in range(4):
        assert ctx.compute(a, b, "se6") == first


def test_barrier_timeout_returns_status(hd):
    # A 1 ns give-up time makes the first waiting CTA abandon the grid barrier:
    # the call must come back with HD_ERR_TIMEOUT and the device stay usable.
    a, b = synth.pair_shifted_union(2, (32, 64, 64), "cuda", rmin=6, rmax=20, max_shift=8)
    with hd.Context(0, barrier_timeout_ns=1) as c:
        with pytest.raises(hd.HDError) as ei:
            c.compute(a, b, "se6")
        assert ei.value.code == hd.HD_ERR_TIMEOUT
    with hd.Context(0) as c:
        r = c.compute(a, b, "se6")
        assert r["status"] == 0 and r["hd"] > 0


def test_iteration_cap(hd):
    a = torch.zeros((8, 8, 64), dtype=torch.uint8, device="cuda")
    b = torch.zeros_like(a)
    a[0, 0, 0] = 1
    b[7, 7, 63] = 1
    with hd.Context(0, max_iterations=5) as c:
        with pytest.raises(hd.HDError) as ei:
            c.compute(a, b, "se6")
        assert ei.value.code == hd.HD_ERR_ITER_LIMIT


def test_bad_arguments(hd, ctx):
    a = torch.zeros((4, 4, 4), dtype=torch.uint8, device="cuda")
    with pytest.raises(ValueError):
        ctx.compute(a, torch.zeros((4, 4, 5), dtype=torch.uint8, device="cuda"))
    with pytest.raises(ValueError):
        ctx.compute(a, a, metric="se26")


def test_reference_class_mirror(hd, oracle):
    a, b = synth.pair_ellipsoid_salt(7)
    a, b = a.numpy(), b.numpy()
    v1, v2 = hd.Volume.from_array(a), hd.Volume.from_array(b)
    h = hd.HausdorffDistance()  # reference default: 18-neighbour element
    assert h.computeDistance(v1, v2) == oracle.forbench(a, b, "se18")["hd"]
    d, avg = hd.HausdorffDistance("se6").computeDistances(v1, v2)
    o = oracle.forbench(a, b, "se6")
    assert d == o["hd"] and avg == o["avg_hd"]
    empty = hd.Volume(64, 64, 64)
    assert h.computeDistance(v1, empty) == -1


def test_context_stream_calls_wait_for_torch_stream(hd, ctx):
    """batch / autotune run on the context's own stream: masks produced on
    torch's stream just before the call must be complete when they are read."""
    from housdorffhdf5cmake_gb300 import synth
    keys = ("hd", "hd_ab", "hd_ba", "sum_ab", "sum_ba", "n_a", "n_b", "status")
    pairs = [synth.pair_shifted_union(900 + i, (192, 256, 256), "cuda", rmin=8, rmax=60, max_shift=9)
             for i in range(3)]
    got = ctx.batch(pairs, "se6")  # no synchronisation between generation and the call
    want = [ctx.compute(a, b, "se6") for a, b in pairs]
    for g, w in zip(got, want):
        assert all(g[k] == w[k] for k in keys), (g, w)
    more = [synth.pair_shifted_union(950, (192, 256, 256), "cuda", rmin=8, rmax=60, max_shift=9)]
    with hd.Context(0) as c:
        c.autotune(more, "se6", repeats=1)  # raises if shapes disagree (a half-written mask would)


def test_async_entry_matches_blocking_entry(hd, ctx):
    """hd_compute_u8_device_async: back-to-back calls on one stream (sizes
    growing and shrinking, both elements, empty masks), results decoded on
    the device, equal field by field to hd_compute_u8_device."""
    import ctypes
    from housdorffhdf5cmake_gb300 import _native as N
    rng = np.random.default_rng(5)
    cases = []
    for i, shape in enumerate([(24, 40, 56), (64, 96, 130), (9, 17, 33), (80, 120, 200), (1, 1, 1)]):
        a, b = random_pair(rng, shape, p_a=0.02, p_b=0.01)
        cases.append((a, b, "se6" if i % 2 == 0 else "se18"))
    z = np.zeros((12, 20, 36), np.uint8)
    one = z.copy()
    one[3, 4, 5] = 1
    cases += [(z, z.copy(), "se6"), (one, z.copy(), "se6"), (one, one.copy(), "se18")]
    a, b = synth.pair_shifted_union(17, (96, 128, 160), "cpu", rmin=6, rmax=40, max_shift=9)
    cases.append((a.numpy(), b.numpy(), "se6"))
    dev = [(cuda(a), cuda(b), m) for a, b, m in cases]
    with hd.Context(0) as c:
        outs = [c.compute_async(a, b, m) for a, b, m in dev]  # no synchronisation in between
        torch.cuda.current_stream().synchronize()
        got = [hd.result_from_bytes(o.cpu()) for o in outs]
        want = [c.compute(a, b, m) for a, b, m in dev]
    for i, (g, w) in enumerate(zip(got, want)):
        for k in w:
            if k == "avg_hd" and w[k] != w[k]:
                assert g[k] != g[k], (i, k)
            else:
                assert g[k] == w[k], (i, k, g, w)
    L = N.load()
    d = cuda(cases[0][0])
    assert L.hd_compute_u8_device_async(ctx.handle, d.data_ptr(), d.data_ptr(), 56, 40, 24, 0, None,
                                        None) == hd.HD_ERR_BAD_ARG


@pytest.mark.parametrize("partitions", [1, 2, 3])
def test_pipelined_entry_matches_blocking_entry(hd, ctx, partitions, monkeypatch):
    """hd_compute_u8_device_pipelined: back-to-back pairs (on split SMs: one
    to three dilation partitions side by side, two workspaces each in turn;
    the 512x512x257 pair is above the split's size limit and runs like
    the asynchronous entry), a blocking call in the middle (which waits for
    the pipelined ones first), results complete after flush(), equal field by
    field to hd_compute_u8_device."""
    from housdorffhdf5cmake_gb300 import _native as N
    monkeypatch.setenv("HD_SPLIT_DILATIONS", str(partitions))  # read when the context first splits
    rng = np.random.default_rng(8)
    cases = []
    for i, shape in enumerate([(24, 40, 56), (64, 96, 130), (9, 17, 33), (80, 120, 200)]):
        a, b = random_pair(rng, shape, p_a=0.02, p_b=0.01)
        cases.append((cuda(a), cuda(b), "se6" if i % 2 == 0 else "se18"))
    for seed, d in ((31, 256), (32, 257)):
        a, b = synth.pair_shifted_union(seed, (d, 512, 512), "cuda", rmin=10, rmax=60, max_shift=12)
        cases.append((a, b, "se6"))
    z = torch.zeros((12, 20, 36), dtype=torch.uint8, device="cuda")
    cases.append((z, z.clone(), "se6"))
    want = [ctx.compute(a, b, m) for a, b, m in cases]
    with hd.Context(0, record_timings=True) as c:
        outs = []
        for rep in range(2):
            for i, (a, b, m) in enumerate(cases):
                outs.append(c.compute_pipelined(a, b, m))
                if rep == 0 and i == 3:  # another call in between waits for the pipelined ones
                    mid = c.compute(*cases[0][:2], cases[0][2])
        c.flush()
        torch.cuda.current_stream().synchronize()
        got = [hd.result_from_bytes(o.cpu()) for o in outs]
        tm = c.last_timings()  # the last pair ran on split SMs
        assert tm["iterations"] == -1 and tm["dilation_partitions"] == partitions, tm
    for k in want[0]:
        assert mid[k] == want[0][k] or (k == "avg_hd" and mid[k] != mid[k])
    for i, g in enumerate(got):
        w = want[i % len(cases)]
        for k in w:
            if k == "avg_hd" and w[k] != w[k]:
                assert g[k] != g[k], (i, k)
            elif k != "iterations":
                assert g[k] == w[k], (i, k, g, w)
    L = N.load()
    assert L.hd_pipeline_flush(None, None) == hd.HD_ERR_BAD_ARG


def test_nonboolean_bytes(hd, ctx, oracle):
    """Foreground = any nonzero byte (forBench/Volume.h's bool masks are one
    byte per voxel): masks whose foreground bytes take values 1..255 in
    every tile, and 0/1 masks with one byte per mask raised above 1 (one
    warp of one tile then leaves the 0/1 packing path), give their 0/1
    form's results through the device, host, batched and pipelined entries,
    for both elements; the 0/1 form equals the oracle."""
    rng = np.random.default_rng(29)
    keys = ("hd", "hd_ab", "hd_ba", "sum_ab", "sum_ba", "n_a", "n_b", "n_a_not_b", "n_b_not_a", "status", "hd_robust")
    for shape in ((33, 70, 95), (20, 48, 128)):
        a, b = random_pair(rng, shape, p_a=0.03, p_b=0.02)
        wide_a = (a * rng.integers(1, 256, a.shape)).astype(np.uint8)
        wide_b = (b * rng.integers(1, 256, b.shape)).astype(np.uint8)
        one_a, one_b = a.copy(), b.copy()
        for m, x in ((a, one_a), (b, one_b)):
            idx = np.flatnonzero(m)
            x.flat[idx[len(idx) // 2]] = 0x80 + int(rng.integers(0, 128))
        for metric in ("se6", "se18"):
            want = ctx.compute(cuda(a), cuda(b), metric)
            o = oracle.forbench(a, b, metric)
            assert want["hd"] == o["hd"] and want["sum_ab"] == o["sum_ab"] and want["sum_ba"] == o["sum_ba"]
            for va, vb in ((wide_a, wide_b), (one_a, one_b)):
                got = [ctx.compute(cuda(va), cuda(vb), metric), ctx.compute(va, vb, metric),
                       ctx.batch([(cuda(va), cuda(vb)), (cuda(a), cuda(b))], metric)[0]]
                with hd.Context(0) as c:
                    o_ = c.compute_pipelined(cuda(va), cuda(vb), metric)
                    c.flush()
                    torch.cuda.current_stream().synchronize()
                    got.append(hd.result_from_bytes(o_.cpu()))
                for g in got:
                    for k in keys:
                        assert g[k] == want[k], (shape, metric, k, g, want)


def test_label_selection(hd, ctx, oracle):
    """label option (the reference's numberToLookFor): a voxel is foreground
    iff its byte equals the label; results equal the binary path on the
    thresholded masks, for device, host and batched inputs and the maps."""
    a, b = synth.pair_shifted_union(23, (40, 72, 100), "cpu", rmin=5, rmax=25, max_shift=7)
    a, b = a.numpy(), b.numpy()
    rng = np.random.default_rng(13)
    va = np.where(a != 0, 3, np.where(rng.random(a.shape) < 0.05, 1, 0)).astype(np.uint8)
    vb = np.where(b != 0, 3, np.where(rng.random(b.shape) < 0.05, 7, 0)).astype(np.uint8)
    keys = ("hd", "hd_ab", "hd_ba", "sum_ab", "sum_ba", "n_a", "n_b", "n_a_not_b", "n_b_not_a", "status", "hd_robust")
    for label in (3, 1):
        ta, tb = (va == label).astype(np.uint8), (vb == label).astype(np.uint8)
        for metric in ("se6", "se18"):
            want = ctx.compute(cuda(ta), cuda(tb), metric)
            o = oracle.forbench(ta, tb, metric)
            assert want["hd"] == o["hd"] and want["sum_ab"] == o["sum_ab"]
            with hd.Context(0, label=label) as c:
                for got in (c.compute(cuda(va), cuda(vb), metric), c.compute(va, vb, metric),
                            c.batch([(cuda(va), cuda(vb))], metric)[0]):
                    for k in keys:
                        assert got[k] == want[k], (label, metric, k, got, want)
                if metric == "se6":
                    _, ma, mb = c.distance_map(cuda(va), cuda(vb), metric)
                    _, wa, wb = ctx.distance_map(cuda(ta), cuda(tb), metric)
                    assert torch.equal(ma, wa) and torch.equal(mb, wb)
    with pytest.raises(hd.HDError):
        hd.Context(0, label=256)


def test_async_host_entry_pipelines_copies(hd, ctx):
    """hd_compute_u8_async: host masks (pinned and pageable) copied on the copy
    stream into alternating staging buffers while earlier pairs compute;
    every result equals the blocking host entry's."""
    rng = np.random.default_rng(21)
    cases = []
    for i, shape in enumerate([(30, 50, 70), (64, 96, 130), (12, 20, 36), (80, 120, 200), (64, 96, 130)]):
        a, b = random_pair(rng, shape, p_a=0.02, p_b=0.01)
        cases.append((a, b, "se6" if i % 2 == 0 else "se18"))
    one = np.zeros((12, 20, 36), np.uint8)
    one[3, 4, 5] = 1
    cases.append((one, np.zeros_like(one), "se6"))
    host = []
    for i, (a, b, m) in enumerate(cases):
        if i % 2 == 0:
            host.append((torch.from_numpy(a).pin_memory(), torch.from_numpy(b).pin_memory(), m))
        else:
            host.append((a, b, m))
    with hd.Context(0) as c:
        outs = [c.compute_async(a, b, m) for a, b, m in host]
        torch.cuda.current_stream().synchronize()
        got = [hd.result_from_bytes(o.cpu()) for o in outs]
        want = [c.compute(a, b, m) for a, b, m in cases]
    for i, (g, w) in enumerate(zip(got, want)):
        for k in w:
            if k == "avg_hd" and w[k] != w[k]:
                assert g[k] != g[k], (i, k)
            else:
                assert g[k] == w[k], (i, k, g, w)


def test_autotune_table_round_trip(hd, tmp_path):
    """The autotuner searches shapes and the queue schedule, writes its table,
    and a new context created with that table runs the tuned shape for the
    same workload class with the same results."""
    import json
    specs = synth.batch_ragged_specs(41, n=20, lo=32, hi=96, edge_frac=0.1)
    pairs = [synth.pair_from_spec(s, "cuda") for s in specs]
    path = str(tmp_path / "tune.json")
    with hd.Context(0, tuning_table=path) as c:
        rep = c.autotune(pairs, "se6", repeats=3)
        first = c.batch(pairs, "se6")
    assert "order=1" in rep and "spread=1" in rep  # the queue schedule was searched
    best = [ln for ln in rep.splitlines() if ln.startswith("best ")]
    assert len(best) == 1
    table = json.load(open(path))["entries"]
    assert len(table) == 1
    (key, entry), = table.items()
    assert best[0].startswith(f"best {key}:")
    for k in ("kernel", "bz", "steps", "ctas_per_sm", "order", "spread"):
        assert f"{k if k != 'ctas_per_sm' else 'cps'}={entry[k]}" in best[0]
    with hd.Context(0, tuning_table=path, record_timings=True) as c2:
        again = c2.batch(pairs, "se6")
        t = c2.last_timings()
    assert t["kernel"] == entry["kernel"] and t["brick_z"] == entry["bz"]
    if entry["kernel"] == 2:
        assert t["steps_per_barrier"] == entry["steps"]
    keys = [k for k in first[0] if k != "iterations"]
    for x, y in zip(first, again):
        assert all(x[k] == y[k] or (k == "avg_hd" and x[k] != x[k] and y[k] != y[k]) for k in keys)


def test_prepared_batch_columns_equal_batch(hd, ctx):
    """A prepared batch run twice (columns and dicts) equals batch()."""
    specs = synth.batch_ragged_specs(43, n=12, lo=24, hi=80, edge_frac=0.2)
    pairs = [synth.pair_from_spec(s, "cuda") for s in specs]
    want = ctx.batch(pairs, "se6")
    prep = ctx.prepare_batch(pairs, "se6")
    assert len(prep) == 12
    for _ in range(2):
        cols = prep.run(columns=True)
        got = prep.run()
        for i, w in enumerate(want):
            for k in KEYS:
                assert got[i][k] == w[k] and int(cols[k][i]) == w[k], (i, k)
    assert ctx.prepare_batch([], "se6").run(columns=True)["hd"].shape == (0,)


@pytest.mark.parametrize("kernel", [1, 2])
def test_se18_paths_that_leave_the_bounding_box(hd, oracle, kernel):
    """The 18-neighbour element's shortest paths may step one voxel out of
    the bounding box of A u B (offset (0, 2, 2) takes the corners (1, 1, 1)
    and (-1, 1, 1)); the CUDA path's domain keeps that margin.  Single voxels
    at such offsets in the middle of the volume, against its faces (where the
    volume clips the margin) and in its corners, thin diagonal lines: every
    field against the oracle's transforms over the whole volume."""
    rng = np.random.default_rng(23)
    cases = []
    V = (12, 40, 70)  # D, H, W: x spans three words
    for (dz, dy, dx) in [(0, 2, 2), (2, 0, 2), (2, 2, 0), (0, 3, 3), (3, 1, 0), (1, 0, 3), (2, 1, 1), (4, 0, 0),
                         (0, 0, 4), (3, 3, 1)]:
        for (z, y, x) in [(5, 20, 35), (0, 0, 0), (0, 20, 31), (5, 0, 32), (10, 38, 64), (7, 39, 69)]:
            zb, yb, xb = z + dz, y + dy, x + dx
            if not (0 <= zb < V[0] and 0 <= yb < V[1] and 0 <= xb < V[2]):
                zb, yb, xb = z - dz, y - dy, x - dx
            if not (0 <= zb < V[0] and 0 <= yb < V[1] and 0 <= xb < V[2]):
                continue
            a = np.zeros(V, np.uint8)
            b = np.zeros(V, np.uint8)
            a[z, y, x] = 1
            b[zb, yb, xb] = 1
            cases.append((a, b))
    for _ in range(12):
        a = np.zeros(V, np.uint8)
        b = np.zeros(V, np.uint8)
        for m in (a, b):
            z, y, x = (int(rng.integers(0, s)) for s in V)
            sz, sy = int(rng.integers(-1, 2)), int(rng.integers(-1, 2))
            for t in range(int(rng.integers(1, 9))):
                if 0 <= z + sz * t < V[0] and 0 <= y + sy * t < V[1]:
                    m[z + sz * t, y + sy * t, x] = 1
        cases.append((a, b))
    with hd.Context(0, kernel=kernel) as kctx:
        for i, (a, b) in enumerate(cases):
            o = oracle.bfs_pair(a, b, "se18")
            assert_same(kctx.compute(cuda(a), cuda(b), "se18"), o, f"case {i} kernel {kernel}")
