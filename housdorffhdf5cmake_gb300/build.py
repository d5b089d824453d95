"""Build recipe of libhd_gb300.so (nvcc, sm_103a only, in-tree, no cmake).

Every .cu / .cpp under csrc/ is compiled to an object in parallel and linked
into ``housdorffhdf5cmake_gb300/_build/libhd_gb300.so`` with the CUDA runtime
linked statically.  Objects are rebuilt only when a source or header changed.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
OBJ = os.path.join(BUILD, "obj")
LIB = os.path.join(BUILD, "libhd_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          f"-I{INCLUDE}", f"-I{CSRC}"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libhd_gb300.so")
    return path


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
            glob.glob(os.path.join(INCLUDE, "hd", "*.h")))


def _compile(src: str, newest_header: float, extra) -> str:
    obj = os.path.join(OBJ, os.path.basename(src) + (".hdf5.o" if "-DHD_WITH_HDF5" in extra else ".o"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), newest_header):
        return obj
    tmp = obj + f".tmp{os.getpid()}"
    cmd = [nvcc(), *ARCH, *CFLAGS, *extra, "-c", src, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, obj)
    return obj


def build(verbose: bool = False, extra_flags=None) -> str:
    """Compile and link the library; returns the path of the .so.

    HD_WITH_HDF5=1 in the environment compiles the HDF5 entry points against
    HDF5's C library (hdf5.h on the include path, -lhdf5 at the link)."""
    os.makedirs(OBJ, exist_ok=True)
    extra = list(extra_flags or [])
    libs = []
    if os.environ.get("HD_WITH_HDF5") == "1":
        extra.append("-DHD_WITH_HDF5")
        libs.append("-lhdf5")
    srcs = _sources()
    newest = max(os.path.getmtime(h) for h in _headers() + [os.path.abspath(__file__)])
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, newest, extra), srcs))
    stamp = os.path.join(BUILD, "link_inputs.txt")  # relink when the object set changes (HDF5 on / off)
    inputs = "\n".join(objs + libs)
    same = os.path.exists(stamp) and open(stamp).read() == inputs
    if not same or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs, *libs, "-lpthread", "-ldl", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
        with open(stamp, "w") as f:
            f.write(inputs)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra_flags=sys.argv[1:])
