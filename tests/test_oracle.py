"""The CPU oracle against independent methods and the golden fixtures.

or_forbench restates forBench/HausdorffDistance.cu:101-187; it must agree with
breadth-first search (any element) and with brute-force nearest-voxel
Manhattan distance (6-neighbour element), on the edge cases the reference's
scenario list (old/testData.cu) names: corners, overlap, distance 1 and 2,
points on block faces, and on ragged shapes.
"""
import numpy as np
import pytest

from housdorffhdf5cmake_gb300 import synth

KEYS = ("hd", "hd_ab", "hd_ba", "sum_ab", "sum_ba", "n_a", "n_b", "n_a_not_b", "n_b_not_a", "status", "avg_hd")


def same(x, y):
    return all((x[k] == y[k]) or (isinstance(x[k], float) and np.isnan(x[k]) and np.isnan(y[k])) for k in KEYS)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_forbench_equals_bfs_and_bruteforce_64(oracle, seed):
    a, b = synth.pair_ellipsoid_salt(seed)
    a, b = a.numpy(), b.numpy()
    f6 = oracle.forbench(a, b, "se6")
    assert same(f6, oracle.bfs_pair(a, b, "se6"))
    assert same(f6, oracle.bruteforce_l1(a, b))
    f18 = oracle.forbench(a, b, "se18")
    assert same(f18, oracle.bfs_pair(a, b, "se18"))
    assert f18["hd"] <= f6["hd"]


@pytest.mark.parametrize("shape", [(1, 1, 1), (1, 1, 9), (1, 13, 1), (11, 1, 1), (1, 17, 23), (5, 7, 33), (9, 9, 64)])
def test_ragged_shapes(oracle, shape):
    rng = np.random.default_rng(sum(shape))
    for p in (0.05, 0.2):
        a = (rng.random(shape) < p).astype(np.uint8)
        b = (rng.random(shape) < p / 2).astype(np.uint8)
        for se in ("se6", "se18"):
            f = oracle.forbench(a, b, se)
            assert same(f, oracle.bfs_pair(a, b, se)), (shape, p, se)
        if a.any() and b.any():
            assert same(oracle.forbench(a, b, "se6"), oracle.bruteforce_l1(a, b))


def test_parallel_equals_serial(oracle):
    a, b = synth.pair_shifted_union(3, (24, 48, 70), "cpu", rmin=4, rmax=15, max_shift=6)
    a, b = a.numpy(), b.numpy()
    for se in ("se6", "se18"):
        assert oracle.forbench(a, b, se, nthreads=1) == oracle.forbench(a, b, se, nthreads=4)


def test_scenarios(oracle):
    """old/testData.cu scenario kinds, re-expressed on a 40x36x33 volume."""
    shape = (33, 36, 40)
    z = np.zeros(shape, np.uint8)
    a, b = z.copy(), z.copy()
    a[0, 0, 0] = 1          # volume corner
    b[0, 0, 1] = 1          # distance 1 (covered by the first dilation)
    r = oracle.forbench(a, b, "se6")
    assert (r["hd"], r["sum_ab"], r["sum_ba"]) == (1, 1, 1)
    b[0, 0, 1] = 0
    b[0, 1, 1] = 1          # distance 2 under SE6, 1 under SE18 (xy diagonal)
    assert oracle.forbench(a, b, "se6")["hd"] == 2
    assert oracle.forbench(a, b, "se18")["hd"] == 1
    b[:] = 0
    b[1, 0, 1] = 1          # xz edge neighbour: not in the 18-element, 2 steps
    assert oracle.forbench(a, b, "se18")["hd"] == 2
    b[:] = 0
    b[1, 1, 1] = 1          # 3D corner: 1 step under SE18, 3 under SE6
    assert oracle.forbench(a, b, "se18")["hd"] == 1
    assert oracle.forbench(a, b, "se6")["hd"] == 3
    # overlap voxels contribute 0 and are not FP/FN
    a[:] = 0
    b[:] = 0
    a[5, 6, 7] = a[9, 11, 7] = 1
    b[5, 6, 7] = b[9, 11, 7] = 1
    r = oracle.forbench(a, b, "se6")
    assert (r["hd"], r["sum_ab"], r["sum_ba"], r["n_a_not_b"]) == (0, 0, 0, 0)
    # far corners of the volume
    a[:] = 0
    b[:] = 0
    a[0, 0, 0] = 1
    b[-1, -1, -1] = 1
    assert oracle.forbench(a, b, "se6")["hd"] == 32 + 35 + 39


def test_empty_masks(oracle):
    z = np.zeros((4, 5, 6), np.uint8)
    one = z.copy()
    one[1, 2, 3] = 1
    r = oracle.forbench(z, z)
    assert r["status"] == 0 and r["hd"] == 0
    r = oracle.forbench(z, one)
    assert r["status"] == oracle.EMPTY and r["hd"] == -1 and np.isnan(r["avg_hd"])
    assert oracle.bfs_pair(one, z)["status"] == oracle.EMPTY


def test_robust_hd_rule(oracle):
    a, b = synth.pair_ellipsoid_salt(4)
    o = oracle.forbench(a.numpy(), b.numpy(), "se6", hist=True)
    assert oracle.robust_hd(o["hist_ab"], o["hist_ba"], o["n_a_not_b"], o["n_b_not_a"], 1.0) == o["hd"]
    r95 = oracle.robust_hd(o["hist_ab"], o["hist_ba"], o["n_a_not_b"], o["n_b_not_a"], 0.95)
    r50 = oracle.robust_hd(o["hist_ab"], o["hist_ba"], o["n_a_not_b"], o["n_b_not_a"], 0.5)
    assert 0 <= r50 <= r95 <= o["hd"]


def test_tile_counts(oracle):
    a = np.zeros((40, 40, 70), np.uint8)
    a[0, 0, 0] = 1
    d = oracle.bfs_dt(a, "se6")
    t = oracle.tile_counts(d, (0, 69, 0, 39, 0, 39), 3)
    assert list(t) == [0, 1, 1, 1]
    t = oracle.tile_counts(d, (0, 69, 0, 39, 0, 39), 40)
    assert t[32] == 4  # distance 32 reaches the x, y and z neighbour tiles and stays in the first


def _crop_margin(a, b, mx, my, mz):
    """The masks on the bounding box of A u B widened by (mx, my, mz) voxels,
    clipped to the volume."""
    u = (a != 0) | (b != 0)
    zz, yy, xx = (np.where(u.any(axis=ax))[0] for ax in ((1, 2), (0, 2), (0, 1)))
    D, H, W = a.shape
    sl = (slice(max(0, zz[0] - mz), min(D, zz[-1] + 1 + mz)), slice(max(0, yy[0] - my), min(H, yy[-1] + 1 + my)),
          slice(max(0, xx[0] - mx), min(W, xx[-1] + 1 + mx)))
    return a[sl].copy(), b[sl].copy()


def _same_pair_result(r, q):
    keys = ("hd", "hd_ab", "hd_ba", "sum_ab", "sum_ba", "n_a", "n_b", "n_a_not_b", "n_b_not_a", "status")
    if any(r[k] != q[k] for k in keys):
        return False
    for h in ("hist_ab", "hist_ba"):
        n = min(len(r[h]), len(q[h]))
        if not np.array_equal(r[h][:n], q[h][:n]) or r[h][n:].any() or q[h][n:].any():
            return False
    return True


def test_se18_domain_margin(oracle):
    """The 18-neighbour domain of the CUDA path is the bounding box of A u B
    widened by one voxel in x and y (the path widens x by a whole word and z
    by a plane as well): on it the breadth-first transforms give the same
    results and per-step histograms as on the whole volume, while the bare
    bounding box does not (a shortest path may step one voxel out of it)."""
    rng = np.random.default_rng(11)
    bare_differs = 0
    cases = 0
    V = 16
    for dz in range(-4, 5):
        for dy in range(-4, 5):
            for dx in range(-4, 5):
                a = np.zeros((V, V, V), np.uint8)
                b = np.zeros_like(a)
                a[8, 8, 8] = 1
                b[8 + dz, 8 + dy, 8 + dx] = 1
                full = oracle.bfs_pair(a, b, "se18", hist=True)
                assert _same_pair_result(full, oracle.bfs_pair(*_crop_margin(a, b, 1, 1, 0), "se18", hist=True)), \
                    (dz, dy, dx)
                bare_differs += not _same_pair_result(full, oracle.bfs_pair(*_crop_margin(a, b, 0, 0, 0), "se18",
                                                                              hist=True))
                cases += 1
    for _ in range(60):
        shape = tuple(int(v) for v in rng.integers(5, 20, size=3))
        p = float(rng.choice([0.003, 0.02, 0.1]))
        a = (rng.random(shape) < p).astype(np.uint8)
        b = (rng.random(shape) < p).astype(np.uint8)
        if not (a.any() and b.any()):
            continue
        full = oracle.bfs_pair(a, b, "se18", hist=True)
        for m in ((1, 1, 0), (1, 1, 1), (32, 1, 1)):
            assert _same_pair_result(full, oracle.bfs_pair(*_crop_margin(a, b, *m), "se18", hist=True)), (shape, m)
        cases += 1
    assert bare_differs > 0  # the margin is needed
