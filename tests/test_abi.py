"""The C ABI library without a GPU: it loads, exports every entry point that
include/hd/hd.h declares, its struct layouts match the Python binding, and the
C++ drop-in header compiles against it."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "hd", "hd.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hd_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(hd):
    from housdorffhdf5cmake_gb300 import _native
    L = _native.load()
    names = declared_functions()
    assert len(names) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", _native.lib_path()], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT (hd_[a-z0-9_]+)$", out, flags=re.M))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    assert sorted(_native.EXPORTS) == names
    for n in names:
        getattr(L, n)


def test_status_strings_and_version(hd):
    from housdorffhdf5cmake_gb300 import _native
    for code in range(11):
        assert _native.status_string(code) not in ("", "unknown status")
    assert _native.status_string(99) == "unknown status"
    assert b"sm_103a" in _native.load().hd_version()


def test_options_defaults(hd):
    from housdorffhdf5cmake_gb300 import _native
    o = _native.HdOptions()
    o.percentile = -1
    _native.load().hd_options_init(ctypes.byref(o))
    assert abs(o.percentile - 0.95) < 1e-7 and o.zero_copy == 1 and o.brick_x_words == 0
    s = _native.HdServerOptions()
    _native.load().hd_server_options_init(ctypes.byref(s))
    assert s.hbm_budget_bytes == 120 << 30 and s.tick_iterations == 64 and s.max_queue == 4096


def test_struct_layouts_match_binding(tmp_path, hd):
    from housdorffhdf5cmake_gb300 import _native as N
    exe = tmp_path / "abi_layout"
    subprocess.run(["gcc", "-std=c11", f"-I{ROOT}/include", "-o", str(exe),
                    os.path.join(ROOT, "tests", "cpp", "abi_layout.c")], check=True)
    lines = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = dict(l.rsplit(" ", 1) for l in lines if l)
    types = {"hd_result": N.HdResult, "hd_options": N.HdOptions, "hd_timings": N.HdTimings,
             "hd_pair_desc": N.HdPairDesc, "hd_server_options": N.HdServerOptions,
             "hd_server_stats": N.HdServerStats}
    for key, val in got.items():
        if "." in key:
            t, m = key.split(".")
            assert getattr(types[t], m).offset == int(val), key
        else:
            assert ctypes.sizeof(types[key]) == int(val), key


def test_cpp_drop_in_header_compiles(tmp_path, hd):
    from housdorffhdf5cmake_gb300 import _native
    lib = _native.lib_path()
    exe = tmp_path / "drop_in"
    subprocess.run(["g++", "-std=c++17", f"-I{ROOT}/include/hd", f"-I{ROOT}/include",
                    os.path.join(ROOT, "tests", "cpp", "drop_in_example.cpp"), "-o", str(exe),
                    f"-L{os.path.dirname(lib)}", "-lhd_gb300", f"-Wl,-rpath,{os.path.dirname(lib)}"], check=True)
    assert exe.exists()


def test_hdf5_loader_reports_unsupported(hd):
    with pytest.raises(hd.HDError) as ei:
        hd.load_hdf5_bool("/nonexistent.h5", "onlyLungsBoolFlat")
    assert ei.value.code in (hd.HD_ERR_UNSUPPORTED, hd.HD_ERR_BAD_ARG)


def test_hdf5_pair_entry_without_hdf5(hd):
    """hd_compute_hdf5 answers HD_ERR_UNSUPPORTED in a build without HDF5 (no
    GPU touched); with HDF5 it validates its arguments first."""
    from housdorffhdf5cmake_gb300 import _native as N
    r = N.HdResult()
    code = N.load().hd_compute_hdf5(None, b"/nonexistent.h5", b"a", b"/nonexistent.h5", b"b", 4, 4, 4, 0,
                                    ctypes.byref(r))
    assert code in (hd.HD_ERR_UNSUPPORTED, hd.HD_ERR_BAD_ARG)


def test_context_without_gpu_fails_cleanly(hd):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(hd.HDError) as ei:
        hd.Context(0)
    assert ei.value.code in (hd.HD_ERR_CUDA, hd.HD_ERR_BAD_ARG)
