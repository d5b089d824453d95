"""The reference's own dilation kernel as a parity pin (test infrastructure).

build() compiles, when the reference sources are present (this container),
forBench/HausdorffDistance.cu from where it lies under /root/reference to PTX
(oracle/_ref/forbench_dilate.ptx, the shipped macros: IS_3D 1, CHEBYSHEV 1 =
the 18-neighbour element), and on any machine with nvcc the driver-API
harness oracle/ref_kernel.cpp into oracle/_build/libref_kernel.so.  The PTX
is text and travels with the repository snapshot to the GPU machine, where
the driver compiles it for the GPU at load time.  Nothing of the reference is
copied into the repository; oracle/_ref is git-ignored.

ref_hd(a, b) then runs the reference kernel under the host loop of
forBench/HausdorffDistance.cu:146-172 and returns its HD.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SRC = "/root/reference/forBench/HausdorffDistance.cu"
PTX = os.path.join(HERE, "_ref", "forbench_dilate.ptx")
HARNESS_SRC = os.path.join(HERE, "ref_kernel.cpp")
HARNESS = os.path.join(HERE, "_build", "libref_kernel.so")

_lib = None


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def build() -> None:
    os.makedirs(os.path.dirname(PTX), exist_ok=True)
    os.makedirs(os.path.dirname(HARNESS), exist_ok=True)
    if os.path.exists(REF_SRC) and (not os.path.exists(PTX) or os.path.getmtime(PTX) < os.path.getmtime(REF_SRC)):
        tmp = PTX + f".tmp{os.getpid()}"
        subprocess.run(["nvcc", "-ptx", "-arch=compute_103a", "-O3", "-w", "-o", tmp, REF_SRC], check=True)
        os.replace(tmp, PTX)
    home = _cuda_home()
    inc = os.path.join(home, "include")
    if not os.path.exists(HARNESS) or os.path.getmtime(HARNESS) < os.path.getmtime(HARNESS_SRC):
        tmp = HARNESS + f".tmp{os.getpid()}"
        libdirs = [os.path.join(home, d) for d in ("lib64", "lib", "lib64/stubs", "lib/stubs", "targets/sbsa-linux/lib/stubs",
                                                   "targets/x86_64-linux/lib/stubs")]
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", f"-I{inc}", "-o", tmp, HARNESS_SRC]
        cmd += [f"-L{d}" for d in libdirs if os.path.isdir(d)] + ["-lcuda"]
        subprocess.run(cmd, check=True)
        os.replace(tmp, HARNESS)


def available() -> bool:
    return os.path.exists(PTX)


def _load():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(HARNESS)
        L.ref_forbench_hd.restype = ctypes.c_int
        L.ref_forbench_hd.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        _lib = L
    return _lib


def ref_hd(a, b, max_trips: int | None = None) -> int:
    """HD of the reference's own kernel (18-neighbour element) on (D, H, W) masks."""
    a = np.ascontiguousarray(a, dtype=np.uint8)
    b = np.ascontiguousarray(b, dtype=np.uint8)
    D, H, W = a.shape
    if max_trips is None:
        max_trips = W + H + D + 3
    out = ctypes.c_int(-1)
    rc = _load().ref_forbench_hd(PTX.encode(), a.ctypes.data, b.ctypes.data, W, H, D, max_trips, ctypes.byref(out))
    if rc == 1:
        raise ValueError("exactly one mask is empty: the reference would loop forever; not run")
    if rc != 0:
        raise RuntimeError(f"reference kernel harness failed: {rc}")
    return int(out.value)
