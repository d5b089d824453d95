"""The oracle against golden HDs produced by the reference's own kernel
(tests/golden/reference_hd.json, written by tests/golden/make_golden.py on a
GPU).  Runs on the CPU: the masks are regenerated from their seeds and
checked against the stored checksums first."""
import json
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
GOLDEN = os.path.join(HERE, "golden", "reference_hd.json")

from cases import cases, checksum  # noqa: E402


@pytest.mark.skipif(not os.path.exists(GOLDEN), reason="golden vectors not generated yet")
def test_oracle_matches_reference_kernel_golden(oracle):
    gold = json.load(open(GOLDEN))["cases"]
    made = cases()
    assert set(gold) == set(made)
    for name, make in made.items():
        a, b = make()
        g = gold[name]
        cs = checksum(a, b)
        for k in ("n_a", "n_b", "crc_a", "crc_b", "shape"):
            assert cs[k] == g[k], (name, k)
        for se in ("se6", "se18"):
            assert oracle.forbench(a, b, se)["hd"] == g[f"hd_{se}"], (name, se)
