"""The C++ drop-in (include/hd/HausdorffDistance.h) at the reference's call
site shape, run on the GPU and checked against the oracle."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_drop_in_runs(tmp_path, hd, oracle):
    from housdorffhdf5cmake_gb300 import _native
    lib = _native.lib_path()
    exe = tmp_path / "drop_in"
    subprocess.run(["g++", "-std=c++17", f"-I{ROOT}/include/hd", f"-I{ROOT}/include",
                    os.path.join(ROOT, "tests", "cpp", "drop_in_example.cpp"), "-o", str(exe),
                    f"-L{os.path.dirname(lib)}", "-lhd_gb300", f"-Wl,-rpath,{os.path.dirname(lib)}"], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    hd_s, avg_s = out.split()[1], out.split()[3]
    W, H, D = 70, 50, 40
    z, y, x = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    a = (((x - 30) ** 2 + (y - 25) ** 2 + (z - 20) ** 2) <= 100).astype(np.uint8)
    b = (((x - 37) ** 2 + (y - 22) ** 2 + (z - 18) ** 2) <= 64).astype(np.uint8)
    o = oracle.forbench(a, b, "se18")  # CHEBYSHEV 1, the reference default
    assert int(hd_s) == o["hd"]
    assert float(avg_s) == o["avg_hd"]
