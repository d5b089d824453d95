"""The reference's own dilation kernel as a parity pin (test infrastructure).

build() compiles, when the reference sources are present (the directory named
by the HD_REFERENCE_ROOT environment variable, else ../reference beside this
repository), forBench/HausdorffDistance.cu from where it lies to PTX
twice, once per structuring element the reference's switches select
(forBench/HausdorffDistance.cuh:7-8):
  oracle/_ref/forbench_se18.ptx  as shipped: IS_3D 1, CHEBYSHEV 1
  oracle/_ref/forbench_se6.ptx   CHEBYSHEV 0: a forced include first includes
                                 the reference header (it is `#pragma once`,
                                 so the .cu's own include of it is skipped)
                                 and then redefines the macro to 0
and, on any machine with nvcc, the driver-API harness oracle/ref_kernel.cpp
into oracle/_build/libref_kernel.so.  The PTX is text and travels with the
repository snapshot to the GPU machine, where the driver compiles it for the
GPU at load time.  Nothing of the reference is copied into the repository;
oracle/_ref is git-ignored.

ref_hd(a, b, se) then runs the reference kernel under the host loop of
forBench/HausdorffDistance.cu:146-172 and returns its HD.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("HD_REFERENCE_ROOT") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
REF_DIR = os.path.join(REF_ROOT, "forBench")
REF_SRC = os.path.join(REF_DIR, "HausdorffDistance.cu")
PTX = {"se18": os.path.join(HERE, "_ref", "forbench_se18.ptx"),
       "se6": os.path.join(HERE, "_ref", "forbench_se6.ptx")}
HARNESS_SRC = os.path.join(HERE, "ref_kernel.cpp")
HARNESS = os.path.join(HERE, "_build", "libref_kernel.so")

_lib = None


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def build() -> None:
    refdir = os.path.join(HERE, "_ref")
    os.makedirs(refdir, exist_ok=True)
    os.makedirs(os.path.dirname(HARNESS), exist_ok=True)
    if os.path.exists(REF_SRC):
        for se, out in PTX.items():
            if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(REF_SRC):
                continue
            cmd = ["nvcc", "-ptx", "-arch=compute_103a", "-O3", "-w"]
            if se == "se6":
                force = os.path.join(refdir, "chebyshev0.h")
                with open(force, "w") as f:
                    f.write(f'#include "{os.path.join(REF_DIR, "HausdorffDistance.cuh")}"\n'
                            "#undef CHEBYSHEV\n#define CHEBYSHEV 0\n")
                cmd += ["-include", force]
            tmp = out + f".tmp{os.getpid()}"
            subprocess.run(cmd + ["-o", tmp, REF_SRC], check=True)
            os.replace(tmp, out)
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


def available(se: str = "se18") -> bool:
    return os.path.exists(PTX[se])


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


def ref_hd(a, b, se: str = "se18", max_trips: int | None = None) -> int:
    """HD of the reference's own kernel on (D, H, W) masks; se = "se18" (the
    shipped CHEBYSHEV 1) or "se6" (CHEBYSHEV 0)."""
    a = np.ascontiguousarray(a, dtype=np.uint8)
    b = np.ascontiguousarray(b, dtype=np.uint8)
    D, H, W = a.shape
    if max_trips is None:
        max_trips = W + H + D + 3
    out = ctypes.c_int(-1)
    rc = _load().ref_forbench_hd(PTX[se].encode(), a.ctypes.data, b.ctypes.data, W, H, D, max_trips,
                                 ctypes.byref(out))
    if rc == 1:
        raise ValueError("exactly one mask is empty: the reference would loop forever; not run")
    if rc != 0:
        raise RuntimeError(f"reference kernel harness failed: {rc}")
    return int(out.value)
