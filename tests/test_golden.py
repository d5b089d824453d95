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


CONFIGS = os.path.join(HERE, "golden", "configs.json")


def test_config_fixtures_cover_every_workload():
    """configs.json holds both 512x512x256 pairs and the 512^3 pair for both
    elements, all 256 ragged pairs and the 48-pair serving pool."""
    cfg = json.load(open(CONFIGS))["configs"]
    assert sorted(cfg["c2"]) == ["pair0_seed1234", "pair1_seed1235"]
    for name in cfg["c2"]:
        assert set(cfg["c2"][name]) == {"se6", "se18"}
        assert all(e["forbench_checked"] for e in cfg["c2"][name].values())
    assert set(cfg["c3"]["far_blobs_seed5"]) == {"se6", "se18"}
    assert cfg["c3"]["far_blobs_seed5"]["se6"]["hd"] >= 200
    assert len(cfg["c4"]) == 256 and len(cfg["c5"]) == 48
    kinds = [e["se6"]["status"] for e in cfg["c4"].values()]
    assert kinds.count(1) >= 5  # the one-sided empty edge pairs


@pytest.mark.parametrize("name", ["pair172", "pair194", "pair069"])
def test_config_fixture_entries_reproduce(oracle, name):
    """The smallest ragged pairs: regenerated on the CPU, same checksums, and
    the oracle's restatement of the reference loop gives the stored result."""
    from make_config_golden import FIELDS, make_masks
    e = json.load(open(CONFIGS))["configs"]["c4"][name]["se6"]
    a, b = (m.numpy() for m in make_masks(tuple(e["key"])))
    cs = checksum(a, b)
    for k in ("n_a", "n_b", "crc_a", "crc_b", "shape"):
        assert cs[k] == e[k], (name, k)
    o = oracle.forbench(a, b, "se6", nthreads=4)
    for k in FIELDS:
        if k != "avg_hd":
            assert o[k] == e[k], (name, k)
    if e["status"] == 0:
        assert o["avg_hd"] == e["avg_hd"]
