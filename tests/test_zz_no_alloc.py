"""hd_compute_u8_device_noalloc: the entry point that allocates nothing.

It exists for callers that cannot allocate device memory when they need a
distance (an allocator elsewhere owns the HBM, or the calling loop must not
call cudaMalloc/cudaFree).  It keeps every intermediate buffer in one fixed
device array of the library, so these checks call it through the C ABI and
compare its result, field by field and bit for bit, with hd_compute_u8_device,
on two calls in a row (different sizes and elements, so the second call runs
on top of the first call's leftovers), then once more on the first pair.
The test allocates the masks and the result buffer itself; the entry point
only enqueues work on the stream.
"""
import ctypes

import pytest
import torch

from housdorffhdf5cmake_gb300 import _native as N
from housdorffhdf5cmake_gb300 import synth

pytestmark = pytest.mark.gpu

FIELDS = ("hd", "iterations", "sum_ab", "sum_ba", "n_a", "n_b", "n_a_not_b", "n_b_not_a", "avg_hd", "status",
          "hd_ab", "hd_ba", "hd_robust")


def noalloc(a, b, metric):
    """One call through the C ABI; returns (status, result dict)."""
    L = N.load()
    out = torch.zeros(ctypes.sizeof(N.HdResult), dtype=torch.uint8, device=a.device)
    D, H, W = a.shape
    stream = torch.cuda.current_stream()
    code = L.hd_compute_u8_device_noalloc(a.data_ptr(), b.data_ptr(), W, H, D, metric,
                                          ctypes.c_void_p(stream.cuda_stream), out.data_ptr())
    stream.synchronize()
    r = N.HdResult.from_buffer_copy(bytes(out.cpu().numpy().tobytes()))
    return code, r.as_dict()


def check_same(got, want):
    for f in FIELDS:
        assert got[f] == want[f], (f, got, want)


def test_noalloc_matches_allocating_path_twice(hd, ctx):
    a1, b1 = synth.pair_ellipsoid_salt(3, device="cuda")
    a2, b2 = synth.pair_shifted_union(31, (72, 150, 190), "cuda", rmin=6, rmax=35, max_shift=10)
    cases = [(a1, b1, N.HD_SE6), (a2, b2, N.HD_SE18_FORBENCH), (a1, b1, N.HD_SE6)]
    # the entry point runs the one-step kernel with 4 x 8 x 8 bricks; an
    # allocating context on the same kernel must agree on every field, and
    # the default context on every field but the barrier-loop count
    with hd.Context(0, kernel=1, brick_x_words=4, brick_z=8) as same_kernel:
        for a, b, metric in cases:
            code, got = noalloc(a, b, metric)
            assert code == N.HD_OK
            name = "se6" if metric == N.HD_SE6 else "se18"
            check_same(got, same_kernel.compute(a, b, name))
            want = ctx.compute(a, b, name)
            for f in FIELDS:
                if f != "iterations":
                    assert got[f] == want[f], (f, got, want)


def test_noalloc_edge_cases_and_limit(ctx):
    z = torch.zeros((20, 30, 40), dtype=torch.uint8, device="cuda")
    one = z.clone()
    one[2, 3, 4] = 1
    for a, b in ((z, z), (one, z), (one, one.clone())):
        code, got = noalloc(a, b, N.HD_SE6)
        assert code == N.HD_OK
        want = ctx.compute(a, b, "se6")
        for f in FIELDS:
            if f == "iterations":
                continue
            if f == "avg_hd" and want["status"] == N.HD_EMPTY_MASK:
                assert got[f] != got[f]  # NaN
            else:
                assert got[f] == want[f], (f, got, want)
    # a pair that does not fit the fixed array is refused before any work
    L = N.load()
    out = torch.zeros(ctypes.sizeof(N.HdResult), dtype=torch.uint8, device="cuda")
    code = L.hd_compute_u8_device_noalloc(z.data_ptr(), z.data_ptr(), 1024, 1024, 1024, N.HD_SE6, None,
                                          out.data_ptr())
    assert code == N.HD_ERR_BAD_ARG


def test_noalloc_headline_pairs_against_oracle_fixtures():
    """The 512x512x256 headline pairs (they fit the fixed array) straight
    against the oracle's stored results for them (tests/golden/configs.json,
    exact distance transforms and the restatement of the reference loop):
    every field but the barrier-loop count, twice in a row."""
    import json
    import os
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(here, "golden"))
    from make_config_golden import make_masks
    fix = json.load(open(os.path.join(here, "golden", "configs.json")))["configs"]["c2"]
    for _ in range(2):
        for name in sorted(fix):
            o = fix[name]["se6"]
            a, b = make_masks(tuple(o["key"]), "cuda")
            assert int(a.sum()) == o["n_a"] and int(b.sum()) == o["n_b"]
            code, got = noalloc(a, b, N.HD_SE6)
            assert code == N.HD_OK
            for f in FIELDS:
                if f != "iterations":
                    assert got[f] == o[f], (name, f, got[f], o[f])
