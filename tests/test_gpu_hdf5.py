"""The reference's HDF5 host path (hd_compute_hdf5): two flat boolean
datasets -> one pair -> the same result as the masks handed over directly.

Runs only where the library was built with HDF5 (HD_WITH_HDF5=1) and h5py
can write the test file; skipped otherwise (neither is available on the
machines this repository is tested on)."""
import numpy as np
import pytest

from housdorffhdf5cmake_gb300 import synth

pytestmark = pytest.mark.gpu


def test_hdf5_pair_equals_direct_call(hd, ctx, tmp_path):
    h5py = pytest.importorskip("h5py")
    a, b = (m.numpy() for m in synth.pair_ellipsoid_salt(3))
    path = str(tmp_path / "masks.hdf5")
    with h5py.File(path, "w") as f:  # flat boolean datasets, as the reference's file holds them
        f.create_dataset("onlyLungsBoolFlat", data=a.reshape(-1).astype(bool))
        f.create_dataset("onlyBladderBoolFlat", data=b.reshape(-1).astype(bool))
    try:
        flat = hd.load_hdf5_bool(path, "onlyLungsBoolFlat")
    except hd.HDError as e:
        if e.code == hd.HD_ERR_UNSUPPORTED:
            pytest.skip("library built without HDF5")
        raise
    assert np.array_equal(flat, a.reshape(-1))
    got = ctx.compute_hdf5(path, "onlyLungsBoolFlat", path, "onlyBladderBoolFlat", a.shape, "se18")
    want = ctx.compute(a, b, "se18")
    assert {k: got[k] for k in want if k != "iterations"} == {k: want[k] for k in want if k != "iterations"}
    with pytest.raises(hd.HDError):
        ctx.compute_hdf5(path, "onlyLungsBoolFlat", path, "onlyBladderBoolFlat", (2, 2, 2), "se18")
