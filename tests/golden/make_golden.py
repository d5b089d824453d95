"""Writes reference_hd.json: the HD that the reference's own `dilate` kernel
(forBench/HausdorffDistance.cu:21-98, compiled from its source to PTX by
oracle/ref_kernel.py) returns under the reference host loop (:146-172), for
every case of cases.py and both structuring elements.

Needs a GPU and oracle/_ref/forbench_se{6,18}.ptx (built where the reference
sources are present).  Usage: python tests/golden/make_golden.py OUT.json
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from cases import cases, checksum  # noqa: E402
from oracle import ref_kernel  # noqa: E402


def main(path):
    out = {"source": "reference dilate kernel (forBench/HausdorffDistance.cu) run on a GPU via oracle/ref_kernel",
           "cases": {}}
    for name, make in cases().items():
        a, b = make()
        entry = checksum(a, b)
        for se in ("se6", "se18"):
            entry[f"hd_{se}"] = ref_kernel.ref_hd(a, b, se)
        out["cases"][name] = entry
        print(name, entry["hd_se6"], entry["hd_se18"], flush=True)
    with open(path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "reference_hd.json"))
