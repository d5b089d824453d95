"""Seeded synthetic mask pairs for the five benchmark workloads.

The reference's own data (512x512x826 lung and bladder masks loaded from an
HDF5 file, forBench/hdf5Manag.cu:196-214) is not public, so every workload here
is synthetic and seeded.  Shapes are ``(D, H, W)`` (z, y, x), x fastest, like
``Volume`` (forBench/Volume.h:51-54).

All arithmetic is integer (int64), and per-voxel randomness comes from an
integer hash of (seed, voxel index), so the same seed gives the same masks on
the CPU and on a GPU.  Per-shape parameters (centres, radii, shifts) come from
numpy's PCG64 generator.

Workloads:
  pair_ellipsoid_salt   64^3, one ellipsoid per mask + 0.1% salt noise
  pair_shifted_union    512x512x256 union of 1-4 ellipsoids, second mask
                        shifted by up to +-15 per axis, 0.5% boundary flips
  pair_far_blobs        512^3, 8 small balls vs 8 balls >= 200 voxels away
  batch_ragged          256 pairs, axes uniform in {64..384}, 5% edge pairs
  serving_stream        Poisson arrivals, log-normal volumes, 10% 512^3
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

_M32 = 0xFFFFFFFF


def _hash32(seed: int, idx: torch.Tensor) -> torch.Tensor:
    """32-bit integer hash of (seed, idx) (low-bias mixer: xor-shift-multiply)."""
    x = (idx * 0x9E3779B1 + (seed * 0x85EBCA77 + 0x165667B1)) & _M32
    x = x ^ (x >> 16)
    x = (x * 0x7FEB352D) & _M32
    x = x ^ (x >> 15)
    x = (x * 0x846CA68B) & _M32
    x = x ^ (x >> 16)
    return x


def _bernoulli(shape, seed: int, p: float, device) -> torch.Tensor:
    D, H, W = shape
    idx = torch.arange(D * H * W, device=device, dtype=torch.int64).view(D, H, W)
    thr = int(p * 4294967296.0)
    return _hash32(seed, idx) < thr


def draw_ellipsoid_into(mask: torch.Tensor, c, r) -> None:
    """Set the voxels of the integer ellipsoid (centre c=(x,y,z), radii r) in mask."""
    D, H, W = mask.shape
    cx, cy, cz = (int(v) for v in c)
    rx, ry, rz = (max(1, int(v)) for v in r)
    x0, x1 = max(0, cx - rx), min(W - 1, cx + rx)
    y0, y1 = max(0, cy - ry), min(H - 1, cy + ry)
    z0, z1 = max(0, cz - rz), min(D - 1, cz + rz)
    if x0 > x1 or y0 > y1 or z0 > z1:
        return
    dev = mask.device
    dx = torch.arange(x0, x1 + 1, device=dev, dtype=torch.int64) - cx
    dy = torch.arange(y0, y1 + 1, device=dev, dtype=torch.int64) - cy
    dz = torch.arange(z0, z1 + 1, device=dev, dtype=torch.int64) - cz
    tx = (dx * ry * rz) ** 2
    ty = (dy * rx * rz) ** 2
    tz = (dz * rx * ry) ** 2
    lim = (rx * ry * rz) ** 2
    inside = (tz.view(-1, 1, 1) + ty.view(1, -1, 1) + tx.view(1, 1, -1)) <= lim
    sub = mask[z0:z1 + 1, y0:y1 + 1, x0:x1 + 1]
    sub |= inside.to(mask.dtype)


def shift_zero_fill(m: torch.Tensor, s) -> torch.Tensor:
    """m shifted by s=(sx,sy,sz) voxels, with zeros shifted in (no wrap-around)."""
    D, H, W = m.shape
    sx, sy, sz = (int(v) for v in s)
    out = torch.zeros_like(m)

    def rng(n, k):
        return (max(0, k), min(n, n + k)), (max(0, -k), min(n, n - k))

    (dx0, dx1), (ox0, ox1) = rng(W, sx)
    (dy0, dy1), (oy0, oy1) = rng(H, sy)
    (dz0, dz1), (oz0, oz1) = rng(D, sz)
    if dx0 < dx1 and dy0 < dy1 and dz0 < dz1:
        out[dz0:dz1, dy0:dy1, dx0:dx1] = m[oz0:oz1, oy0:oy1, ox0:ox1]
    return out


def boundary6(m: torch.Tensor) -> torch.Tensor:
    """Voxels with at least one in-volume 6-neighbour of the opposite value."""
    b = m != 0
    out = torch.zeros_like(b)
    for dim in range(3):
        n = b.shape[dim]
        if n < 2:
            continue
        lo = b.narrow(dim, 0, n - 1)
        hi = b.narrow(dim, 1, n - 1)
        diff = lo != hi
        out.narrow(dim, 0, n - 1).logical_or_(diff)
        out.narrow(dim, 1, n - 1).logical_or_(diff)
    return out


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(int(seed)))


def pair_ellipsoid_salt(seed: int, shape=(64, 64, 64), device="cpu"):
    """Two 64^3 masks: one solid ellipsoid each (centre uniform in the central
    50% box, radii uniform in [6, 20]) plus Bernoulli(0.001) salt set to 1."""
    D, H, W = shape
    g = _rng(seed)
    out = []
    for m in range(2):
        mask = torch.zeros(shape, dtype=torch.uint8, device=device)
        c = [int(g.integers(n // 4, n - n // 4)) for n in (W, H, D)]
        r = [int(g.integers(6, 21)) for _ in range(3)]
        draw_ellipsoid_into(mask, c, r)
        salt = _bernoulli(shape, seed * 2 + m + 1, 0.001, device)
        mask |= salt.to(torch.uint8)
        out.append(mask)
    return out[0], out[1]


def _union_params(g: np.random.Generator, shape, rmin: float, rmax: float):
    D, H, W = shape
    k = int(g.integers(1, 5))
    ells = []
    for _ in range(k):
        c = [int(g.integers(n // 4, max(n // 4 + 1, n - n // 4))) for n in (W, H, D)]
        r = [int(g.integers(int(rmin), int(rmax) + 1)) for _ in range(3)]
        ells.append((c, r))
    return ells


def pair_shifted_union(seed: int, shape=(256, 512, 512), device="cpu", rmin=10, rmax=80,
                       max_shift=15, flip_p=0.005):
    """CT-like pair: A is a union of 1-4 ellipsoids (radii uniform in
    [rmin, rmax]); B is A shifted by up to +-max_shift voxels per axis with
    zeros shifted in, then each boundary voxel of B is flipped with
    probability flip_p."""
    g = _rng(seed)
    a = torch.zeros(shape, dtype=torch.uint8, device=device)
    for c, r in _union_params(g, shape, rmin, rmax):
        draw_ellipsoid_into(a, c, r)
    s = [int(g.integers(-max_shift, max_shift + 1)) for _ in range(3)]
    b = shift_zero_fill(a, s)
    flip = boundary6(b) & _bernoulli(shape, seed * 7 + 3, flip_p, device)
    b ^= flip.to(torch.uint8)
    return a, b


def pair_far_blobs(seed: int, shape=(512, 512, 512), device="cpu", n_blobs=8, rmin=3, rmax=6,
                   min_dist=200.0):
    """Worst case for the frontier queue: A = 8 balls of radius 3-6; B = 8
    balls whose centres are at Euclidean distance >= min_dist from every A
    centre (rejection sampling), so hundreds of dilation steps are needed."""
    D, H, W = shape
    g = _rng(seed)
    a = torch.zeros(shape, dtype=torch.uint8, device=device)
    b = torch.zeros(shape, dtype=torch.uint8, device=device)
    ca = []
    for _ in range(n_blobs):
        r = int(g.integers(rmin, rmax + 1))
        c = [int(g.integers(r, n - r)) for n in (W, H, D)]
        ca.append(c)
        draw_ellipsoid_into(a, c, (r, r, r))
    placed = 0
    tries = 0
    while placed < n_blobs:
        tries += 1
        if tries > 100000:
            raise RuntimeError("could not place far blobs; volume too small for min_dist")
        r = int(g.integers(rmin, rmax + 1))
        c = [int(g.integers(r, n - r)) for n in (W, H, D)]
        if all(math.dist(c, q) >= min_dist for q in ca):
            draw_ellipsoid_into(b, c, (r, r, r))
            placed += 1
    return a, b


@dataclass
class PairSpec:
    """One pair of a ragged batch: shape (D, H, W), seed and edge-case kind."""
    shape: tuple
    seed: int
    kind: str  # "normal" | "empty_b" | "identical"


def batch_ragged_specs(seed: int, n: int = 256, lo: int = 64, hi: int = 384, edge_frac=0.05):
    """Shapes and kinds of the ragged batch: every axis uniform in {lo..hi};
    edge_frac of the pairs are edge cases, half with an empty second mask and
    half with two identical masks."""
    g = _rng(seed)
    specs = []
    n_edge = int(round(n * edge_frac))
    edge_idx = set(int(i) for i in g.choice(n, size=n_edge, replace=False)) if n_edge else set()
    edge_list = sorted(edge_idx)
    for i in range(n):
        shape = tuple(int(g.integers(lo, hi + 1)) for _ in range(3))
        kind = "normal"
        if i in edge_idx:
            kind = "empty_b" if edge_list.index(i) % 2 == 0 else "identical"
        specs.append(PairSpec(shape, seed * 1000003 + i, kind))
    return specs


def pair_from_spec(spec: PairSpec, device="cpu"):
    """Masks of one ragged-batch pair: the shifted-union generator with radii
    and shift scaled to the smallest axis (radii [10,80] and shift 15 belong to
    a 256-voxel axis)."""
    s = min(spec.shape) / 256.0
    rmin = max(2, int(round(10 * s)))
    rmax = max(rmin + 1, int(round(80 * s)))
    shift = max(1, int(round(15 * s)))
    a, b = pair_shifted_union(spec.seed, spec.shape, device, rmin=rmin, rmax=rmax, max_shift=shift)
    if spec.kind == "empty_b":
        b = torch.zeros_like(a)
    elif spec.kind == "identical":
        b = a.clone()
    return a, b


@dataclass
class RequestSpec:
    """One serving request: arrival time (s), shape (D, H, W), seed."""
    t_arrival: float
    shape: tuple
    seed: int


def serving_stream(seed: int, n: int, rate_hz: float, median=(160, 256, 256), sigma=0.35,
                   cap=512, outlier_frac=0.10):
    """Open-loop Poisson stream: exponential inter-arrival times at rate_hz,
    volume scale log-normal around `median` (aspect kept, every axis capped at
    `cap` by scaling all axes together), and outlier_frac of the requests
    forced to cap^3."""
    g = _rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += float(g.exponential(1.0 / rate_hz)) if rate_hz > 0 else 0.0
        if g.random() < outlier_frac:
            shape = (cap, cap, cap)
        else:
            f = float(np.exp(g.normal(0.0, sigma)))
            dims = [max(16, int(round(m * f))) for m in median]
            big = max(dims)
            if big > cap:
                dims = [max(16, int(d * cap / big)) for d in dims]
            shape = tuple(dims)
        out.append(RequestSpec(t, shape, seed * 7919 + i))
    return out


def pair_for_request(req: RequestSpec, device="cpu"):
    return pair_from_spec(PairSpec(req.shape, req.seed, "normal"), device)
