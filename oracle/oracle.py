"""CPU oracle for the dilation-based Hausdorff distance (ctypes wrapper).

TEST INFRASTRUCTURE ONLY: the test suite, the smoke check and the CPU-baseline
leg of ``bench.py`` import this module as the checker.  The library never does.

Masks are numpy ``uint8`` arrays of shape ``(D, H, W)`` in C order, so x is the
fastest axis exactly like ``Volume`` (forBench/Volume.h:51-54, index
``x + W*y + W*H*z``).  Nonzero means foreground.

Functions (C sources in ``hd_oracle.c``):
  forbench(a, b, se, nthreads)  restatement of forBench/HausdorffDistance.cu:101-187
  bfs_dt(src, se)               exact distance transform by breadth-first search
  bfs_pair(a, b, se)            both transforms -> pair result
  bruteforce_l1(a, b)           nearest-voxel Manhattan distance (6-neighbour element)
  tile_counts(dist, box, kmax)  32^3 tiles touched by each dilation step
  robust_hd(hist, total, p)     percentile HD with the stopping rule of hello.cu:1751-1758
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "hd_oracle.c")
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "libhd_oracle.so")

SE6 = 0
SE18 = 1
_SE = {"se6": SE6, "se18": SE18, SE6: SE6, SE18: SE18}

OK, EMPTY, BAD, OOM, ITER = 0, 1, 2, 3, 7


class OrResult(ctypes.Structure):
    _fields_ = [
        ("hd", ctypes.c_int32),
        ("iterations", ctypes.c_int32),
        ("sum_ab", ctypes.c_uint64),
        ("sum_ba", ctypes.c_uint64),
        ("n_a", ctypes.c_uint64),
        ("n_b", ctypes.c_uint64),
        ("n_a_not_b", ctypes.c_uint64),
        ("n_b_not_a", ctypes.c_uint64),
        ("avg_hd", ctypes.c_double),
        ("status", ctypes.c_int32),
        ("hd_ab", ctypes.c_int32),
        ("hd_ba", ctypes.c_int32),
        ("pad", ctypes.c_int32),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "pad"}


_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile hd_oracle.c into oracle/_build/libhd_oracle.so (gcc, OpenMP)."""
    os.makedirs(_BUILD, exist_ok=True)
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(_SRC):
        tmp = _LIB_PATH + f".tmp{os.getpid()}"
        cmd = ["gcc", "-O3", "-std=c11", "-fopenmp", "-fPIC", "-shared", "-o", tmp, _SRC]
        subprocess.run(cmd, check=True)
        os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            u8p = ctypes.POINTER(ctypes.c_uint8)
            i32p = ctypes.POINTER(ctypes.c_int32)
            u64p = ctypes.POINTER(ctypes.c_uint64)
            rp = ctypes.POINTER(OrResult)
            i = ctypes.c_int
            L.or_forbench.argtypes = [u8p, u8p, i, i, i, i, i, rp, u64p, u64p, i]
            L.or_bfs_dt.argtypes = [u8p, i, i, i, i, i32p]
            L.or_bfs_pair.argtypes = [u8p, u8p, i, i, i, i, rp, u64p, u64p, i]
            L.or_hd_from_dt.argtypes = [u8p, u8p, i32p, i32p, i, i, i, rp, u64p, u64p, i]
            L.or_bruteforce_l1.argtypes = [u8p, u8p, i, i, i, rp]
            L.or_tile_counts.argtypes = [i32p, i, i, i, i, i, i, i, i, i, i, u64p]
            for f in ("or_forbench", "or_bfs_dt", "or_bfs_pair", "or_hd_from_dt",
                      "or_bruteforce_l1", "or_tile_counts"):
                getattr(L, f).restype = ctypes.c_int
            _lib = L
    return _lib


def _u8(a) -> np.ndarray:
    a = np.ascontiguousarray(a)
    if a.ndim != 3:
        raise ValueError("masks must have shape (D, H, W)")
    if a.dtype != np.uint8:
        a = (a != 0).astype(np.uint8)
    return a


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def _dims(a):
    D, H, W = a.shape
    return int(W), int(H), int(D)


def _hist_len(a) -> int:
    W, H, D = _dims(a)
    return W + H + D + 3


def forbench(a, b, se="se6", nthreads: int = 1, hist: bool = False) -> dict:
    """Restated reference loop (forBench/HausdorffDistance.cu:146-172)."""
    a, b = _u8(a), _u8(b)
    if a.shape != b.shape:
        raise ValueError("mask shapes differ")
    W, H, D = _dims(a)
    r = OrResult()
    n = _hist_len(a)
    ha = np.zeros(n, np.uint64)
    hb = np.zeros(n, np.uint64)
    lib().or_forbench(_p(a, ctypes.c_uint8), _p(b, ctypes.c_uint8), W, H, D, _SE[se], int(nthreads),
                      ctypes.byref(r), _p(ha, ctypes.c_uint64), _p(hb, ctypes.c_uint64), n)
    out = r.as_dict()
    if hist:
        out["hist_ab"], out["hist_ba"] = ha, hb
    return out


def bfs_dt(src, se="se6") -> np.ndarray:
    src = _u8(src)
    W, H, D = _dims(src)
    dist = np.empty(src.shape, np.int32)
    st = lib().or_bfs_dt(_p(src, ctypes.c_uint8), W, H, D, _SE[se], _p(dist, ctypes.c_int32))
    if st != OK:
        raise RuntimeError(f"or_bfs_dt failed: {st}")
    return dist


def bfs_pair(a, b, se="se6", hist: bool = False) -> dict:
    a, b = _u8(a), _u8(b)
    W, H, D = _dims(a)
    r = OrResult()
    n = _hist_len(a)
    ha = np.zeros(n, np.uint64)
    hb = np.zeros(n, np.uint64)
    lib().or_bfs_pair(_p(a, ctypes.c_uint8), _p(b, ctypes.c_uint8), W, H, D, _SE[se], ctypes.byref(r),
                      _p(ha, ctypes.c_uint64), _p(hb, ctypes.c_uint64), n)
    out = r.as_dict()
    if hist:
        out["hist_ab"], out["hist_ba"] = ha, hb
    return out


def bruteforce_l1(a, b) -> dict:
    a, b = _u8(a), _u8(b)
    W, H, D = _dims(a)
    r = OrResult()
    lib().or_bruteforce_l1(_p(a, ctypes.c_uint8), _p(b, ctypes.c_uint8), W, H, D, ctypes.byref(r))
    return r.as_dict()


def tile_counts(dist: np.ndarray, box, kmax: int) -> np.ndarray:
    """T_k, k = 0..kmax (T_0 = 0): 32^3 tiles with a voxel at distance k inside box.

    box = (x0, x1, y0, y1, z0, z1), inclusive bounds.
    """
    dist = np.ascontiguousarray(dist, dtype=np.int32)
    D, H, W = dist.shape
    counts = np.zeros(kmax + 1, np.uint64)
    x0, x1, y0, y1, z0, z1 = (int(v) for v in box)
    st = lib().or_tile_counts(_p(dist, ctypes.c_int32), W, H, D, x0, x1, y0, y1, z0, z1, int(kmax),
                              _p(counts, ctypes.c_uint64))
    if st != OK:
        raise RuntimeError(f"or_tile_counts failed: {st}")
    return counts


def robust_hd(hist_ab, hist_ba, n_a_not_b: int, n_b_not_a: int, p: float) -> int:
    """Percentile HD following the stopping rule of hello.cu:1751-1758.

    The reference keeps dilating while ``total * robustnessPercent > covered``
    in float32 for either direction, where ``total`` is the number of voxels of
    one mask outside the other (its FP or FN count) and ``covered`` the number
    of them reached so far.  The result is the first k at which both
    directions have stopped (0 when there is nothing to cover).
    """
    pf = np.float32(p)

    def one(hist, total):
        total_f = np.float32(total) * pf
        cov = 0
        for k in range(len(hist)):
            if k > 0:
                cov += int(hist[k])
            if not (total_f > np.float32(cov)):
                return k
        return len(hist) - 1

    return max(one(hist_ab, n_a_not_b), one(hist_ba, n_b_not_a))
