"""Writes configs.json: oracle results for every benchmark workload at its
stated size, so the GPU tests can check the CUDA path against them without
running the CPU oracle on half-gigavoxel pairs.

Workloads (masks from housdorffhdf5cmake_gb300.synth, integer-exact, so the
GPU machine regenerates the same bytes; each entry carries the masks' counts and
CRC32 to detect generator drift):
  c2      the two 512x512x256 CT-like pairs of the headline (seeds 1234,
          1235), 6- and 18-neighbour elements
  c3      the 512^3 far-blobs pair (seed 5), both elements
  c4      all 256 ragged pairs of the batch workload (batch_ragged_specs(77)),
          6-neighbour element
  c5      the 48-pair request pool of the serving workload
          (serving_stream(4242, n=48)), 6-neighbour element

Every value comes from the oracle's breadth-first distance transform
(oracle.bfs_pair: exact d(v, other mask) under the element for every voxel,
hence hd, one-sided hds, the exact sums, counts and the per-step histogram
that the robust HD is read from, with the stopping rule of hello.cu:1751-1758
at p = 0.95).  The C2 pairs are also run through the oracle's restatement of
the reference loop (oracle.forbench, forBench/HausdorffDistance.cu:101-187),
and the two must agree field by field.

Usage: python tests/golden/make_config_golden.py [OUT.json] [--procs N]
"""
import json
import multiprocessing as mp
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, HERE):
    if p not in sys.path:
        sys.path.insert(0, p)

FIELDS = ("hd", "hd_ab", "hd_ba", "sum_ab", "sum_ba", "n_a", "n_b", "n_a_not_b", "n_b_not_a", "avg_hd", "status")
ROBUST_P = 0.95


def workloads():
    """(config, name, element, maker) for every fixture entry; maker() -> (a, b) CPU uint8 tensors."""
    from housdorffhdf5cmake_gb300 import synth
    out = []
    for i in range(2):
        seed = 1234 + i
        for se in ("se6", "se18"):
            out.append(("c2", f"pair{i}_seed{seed}", se,
                        ("shifted_union", seed)))
    for se in ("se6", "se18"):
        out.append(("c3", "far_blobs_seed5", se, ("far_blobs", 5)))
    for i, s in enumerate(synth.batch_ragged_specs(77, n=256)):
        out.append(("c4", f"pair{i:03d}", "se6", ("ragged", i)))
    for i, r in enumerate(synth.serving_stream(4242, n=48, rate_hz=0.0)):
        out.append(("c5", f"req{i:02d}", "se6", ("request", i)))
    return out


def make_masks(key, device="cpu"):
    """The masks of one fixture entry (same generator calls as bench.py)."""
    from housdorffhdf5cmake_gb300 import synth
    kind, arg = key
    if kind == "shifted_union":
        return synth.pair_shifted_union(arg, (256, 512, 512), device)
    if kind == "far_blobs":
        return synth.pair_far_blobs(arg, (512, 512, 512), device)
    if kind == "ragged":
        return synth.pair_from_spec(synth.batch_ragged_specs(77, n=256)[arg], device)
    if kind == "request":
        return synth.pair_for_request(synth.serving_stream(4242, n=48, rate_hz=0.0)[arg], device)
    raise ValueError(kind)


def _one(job):
    cfg, name, se, key = job
    from cases import checksum
    from oracle import oracle as O
    a, b = (m.numpy() for m in make_masks(key))
    r = O.bfs_pair(a, b, se, hist=True)
    entry = checksum(a, b)
    entry.update({k: r[k] for k in FIELDS})
    entry["hd_robust"] = (O.robust_hd(r["hist_ab"], r["hist_ba"], r["n_a_not_b"], r["n_b_not_a"], ROBUST_P)
                          if r["status"] == 0 else -1)
    if cfg == "c2":
        f = O.forbench(a, b, se, nthreads=max(1, os.cpu_count() // 2))
        bad = [k for k in FIELDS if k != "avg_hd" and f[k] != r[k]] + (
            ["avg_hd"] if f["avg_hd"] != r["avg_hd"] else [])
        if bad:
            raise AssertionError(f"{cfg}/{name}/{se}: restatement and BFS differ in {bad}")
        entry["forbench_checked"] = True
    entry["key"] = list(key)
    return cfg, name, se, entry


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    path = args[0] if args else os.path.join(HERE, "configs.json")
    procs = os.cpu_count() or 1
    if "--procs" in sys.argv:
        procs = int(sys.argv[sys.argv.index("--procs") + 1])
    from oracle import oracle as O
    O.build()
    jobs = workloads()
    t0 = time.time()
    out = {"source": "oracle.bfs_pair (exact distance transform; C2 also oracle.forbench), "
                     "robust HD at p = 0.95", "robust_p": ROBUST_P, "configs": {}}
    # heavy entries first so the pool's tail is short
    order = sorted(range(len(jobs)), key=lambda i: jobs[i][0] not in ("c2", "c3"))
    with mp.get_context("spawn").Pool(procs) as pool:
        for cfg, name, se, entry in pool.imap_unordered(_one, [jobs[i] for i in order]):
            out["configs"].setdefault(cfg, {}).setdefault(name, {})[se] = entry
            print(f"{time.time() - t0:7.1f}s {cfg} {name} {se} hd={entry['hd']}", flush=True)
    with open(path, "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
