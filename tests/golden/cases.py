"""Seeded mask pairs of the golden vectors (shared by make_golden.py and the
tests).  Every generator is integer-exact, so the masks are identical on any
machine.  No case has exactly one empty mask: the reference's loop never ends
on those (forBench/HausdorffDistance.cu:96), so they are not run through it."""
import zlib

import numpy as np

from housdorffhdf5cmake_gb300 import synth


def _rand(shape, seed, pa, pb):
    g = np.random.Generator(np.random.PCG64(seed))
    a = (g.random(shape) < pa).astype(np.uint8)
    b = (g.random(shape) < pb).astype(np.uint8)
    a.flat[0] = 1  # never empty
    b.flat[-1] = 1
    return a, b


def _points(shape, pa, pb):
    a = np.zeros(shape, np.uint8)
    b = np.zeros(shape, np.uint8)
    for p in pa:
        a[p] = 1
    for p in pb:
        b[p] = 1
    return a, b


def cases():
    out = {}
    for seed in range(1, 7):
        out[f"ellipsoid_salt_64_seed{seed}"] = lambda s=seed: tuple(m.numpy() for m in synth.pair_ellipsoid_salt(s))
    for i, shape in enumerate([(1, 1, 1), (1, 37, 1), (1, 1, 70), (5, 3, 33), (7, 64, 65), (3, 17, 129), (1, 40, 50),
                               (33, 31, 95), (9, 2, 31), (16, 16, 160)]):
        out[f"random_{shape[0]}x{shape[1]}x{shape[2]}"] = lambda sh=shape, s=100 + i: _rand(sh, s, 0.02, 0.01)
    # old/testData.cu scenario kinds (corners, distance 1 and 2, diagonals, overlap, far corners)
    sh = (33, 36, 40)
    out["scenario_distance1"] = lambda: _points(sh, [(0, 0, 0)], [(0, 0, 1)])
    out["scenario_xy_diagonal"] = lambda: _points(sh, [(0, 0, 0)], [(0, 1, 1)])
    out["scenario_xz_edge"] = lambda: _points(sh, [(0, 0, 0)], [(1, 0, 1)])
    out["scenario_3d_corner"] = lambda: _points(sh, [(0, 0, 0)], [(1, 1, 1)])
    out["scenario_overlap"] = lambda: _points(sh, [(5, 6, 7), (9, 11, 7)], [(5, 6, 7), (9, 11, 7)])
    out["scenario_far_corners"] = lambda: _points(sh, [(0, 0, 0)], [(32, 35, 39)])
    out["scenario_block_faces"] = lambda: _points(sh, [(16, 18, 0), (16, 0, 20), (0, 18, 20)],
                                                  [(16, 18, 39), (16, 35, 20), (32, 18, 20)])
    out["shifted_union_96x160x192"] = lambda: tuple(
        m.numpy() for m in synth.pair_shifted_union(21, (96, 160, 192), "cpu", rmin=8, rmax=40, max_shift=12))
    return out


def checksum(a, b):
    """Counts and CRC32 of both masks (detects generator drift)."""
    return {"n_a": int(a.astype(bool).sum()), "n_b": int(b.astype(bool).sum()),
            "crc_a": zlib.crc32(np.packbits(a.astype(bool)).tobytes()),
            "crc_b": zlib.crc32(np.packbits(b.astype(bool)).tobytes()),
            "shape": list(a.shape)}
