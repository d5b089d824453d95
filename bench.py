#!/usr/bin/env python
"""Benchmark of the GB300 dilation-based Hausdorff distance.

Headline workload (one step = one pair): two 512x512x256 uint8 CT-like masks
(union of 1-4 ellipsoids, second mask shifted by up to +-15 voxels with 0.5%
boundary flips), 6-neighbour element, packed 32 voxels per uint32 along x.
The reference's own data (512x512x826 lung/bladder HDF5 masks) is not
available; the masks are seeded synthetic stand-ins with the stated shapes.

  value  pairs/s with the masks resident in HBM: K pairs enqueued back to
         back through hd_compute_u8_device_pipelined and one flush (packing
         and set-up on a few SMs, consecutive pairs dilating side by side on
         groups of the other SMs; each result decoded on the device and
         checked afterwards), CUDA events on the launch stream around the K
         steps; two distinct pairs alternate so every step reads
         masks that are not in L2 (2 x 134 MB > 126 MB L2).  The blocking
         device entry (hd_compute_u8_device) is reported beside it
  e2e    pairs/s with pinned HOST masks through hd_compute_u8_async: each
         pair's masks are copied over the host link (DMA) while the previous
         pair computes, and each result is read back to the host; the
         blocking hd_compute_u8 (one call per pair) is reported beside it
Extra keys: Gvoxel-iter/s, the roofline of the dominant kernel, the serial
CPU baseline (the oracle's restatement of the reference loop, 1 core), the
ragged 256-pair batch (one persistent launch) against the same pairs one call
each, the 512^3 far-blob worst case of the frontier queue, and a Poisson
serving stream through the continuous-batching server.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun every rank computes its own pair (replicas, weak scaling) and
rank 0 prints one JSON line.  --impl reference times the reference algorithm
on the host cores (the oracle's restatement of forBench/HausdorffDistance.cu
with all host threads) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import shutil
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W_, H_, D_ = 512, 512, 256
WORKLOAD = "plain single pair 512x512x256 uint8, 6-neighbour element (CT-like shifted ellipsoid unions)"


def _dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            with open(self.path) as f:
                for line in f:
                    parts = [p.strip() for p in line.split(",")]
                    if len(parts) >= 9:
                        rows.append(parts)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def bench_ours(args):
    import numpy as np
    import torch

    import housdorffhdf5cmake_gb300 as hd
    from housdorffhdf5cmake_gb300 import synth

    ws, rank, local = _dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    seed = 1234 + 2 * rank
    # two distinct pairs used alternately: each step reads 134 MB of masks the
    # previous step did not touch (268 MB in turn, more than the 126 MB L2)
    pairs = [synth.pair_shifted_union(seed + i, (D_, H_, W_), dev) for i in range(2)]
    a, b = pairs[0]
    N = W_ * H_ * D_
    # every timed region runs on a context without per-kernel timing events;
    # the phase breakdown comes from a second, instrumented context
    ctx = hd.Context(local)
    tctx = hd.Context(local, record_timings=True)
    stream = torch.cuda.current_stream()

    refs = [ctx.compute(x, y, "se6") for x, y in pairs]
    # both pairs against the oracle's results for these masks (every field)
    for i, r in enumerate(refs):
        _check_fixture(r, "c2", f"pair{i}_seed{seed + i}", "se6", f"headline pair {i}")
    # phase times of the blocking entry (CUDA events around each kernel)
    phases, blocking = [], []
    for w in range(max(args.warmup, 4)):
        x, y = pairs[w % 2]
        assert tctx.compute(x, y, "se6") == refs[w % 2], "non-deterministic result"
        phases.append(tctx.last_timings())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = ctx.compute(x, y, "se6")
        e1.record(stream)
        e1.synchronize()
        assert r == refs[w % 2], "non-deterministic result"
        blocking.append(e0.elapsed_time(e1))
    phases = phases[-2:]
    # warm-up of the enqueue-only entries used in the timed regions (the
    # first pipelined calls set up the split SMs and allocate the six
    # workspaces, one per call)
    outs = torch.empty((args.steps, hd.RESULT_BYTES), dtype=torch.uint8, device=dev)
    for w in range(max(args.warmup, 6)):
        x, y = pairs[w % 2]
        ctx.compute_async(x, y, "se6", out=outs[w % args.steps])
        ctx.compute_pipelined(x, y, "se6", out=outs[(w + 1) % args.steps])
    ctx.flush()
    torch.cuda.synchronize()

    # ---- device-resident timed region ---------------------------------------
    # K pairs enqueued back to back through hd_compute_u8_device_pipelined
    # (each result decoded on the device into its own slot; a pair's packing
    # and set-up run beside earlier pairs' dilations, which run side by side
    # on groups of SMs), one flush, one synchronisation
    clocks = ClockSampler(local)
    with clocks:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        wall0 = time.perf_counter()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(args.steps):
            x, y = pairs[k % 2]
            ctx.compute_pipelined(x, y, "se6", out=outs[k])
        ctx.flush()
        e1.record(stream)
        e1.synchronize()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        wall = time.perf_counter() - wall0
    times = [e0.elapsed_time(e1) / args.steps] * args.steps
    host_outs = outs.cpu()
    for k in range(args.steps):
        assert hd.result_from_bytes(host_outs[k]) == refs[k % 2], f"step {k}: result differs"
    # the same K pairs through hd_compute_u8_device_async (each pair waits for
    # the previous one to finish on the stream)
    torch.cuda.synchronize()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for k in range(args.steps):
        x, y = pairs[k % 2]
        ctx.compute_async(x, y, "se6", out=outs[k])
    s1.record(stream)
    s1.synchronize()
    serial_ms = s0.elapsed_time(s1) / args.steps
    host_outs = outs.cpu()
    for k in range(args.steps):
        assert hd.result_from_bytes(host_outs[k]) == refs[k % 2], f"async step {k}: result differs"
    clk = clocks.summary()
    step_ms = sum(times) / len(times)
    if dist:
        t = torch.tensor([step_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        step_ms = float(t.item())
    value = ws * 1000.0 / step_ms

    # ---- end to end through the host API (pinned host masks) ----------------
    # Pipelined: hd_compute_u8_async copies each pair's pinned host masks by
    # DMA on the context's copy stream while the previous pair computes; each
    # step's 64-byte result is read back to pinned host memory on the stream.
    hpairs = [(x.cpu().pin_memory(), y.cpu().pin_memory()) for x, y in pairs]
    rbytes = hd.RESULT_BYTES
    e_outs = torch.empty((args.steps, rbytes), dtype=torch.uint8, device=dev)
    h_outs = torch.empty((args.steps, rbytes), dtype=torch.uint8).pin_memory()
    for w in range(max(args.warmup, 6)):
        ctx.compute_async(*hpairs[w % 2], "se6", out=e_outs[w % args.steps])
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        ctx.compute_async(*hpairs[k % 2], "se6", out=e_outs[k])
        h_outs[k].copy_(e_outs[k], non_blocking=True)
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1000.0 / args.steps
    for k in range(args.steps):
        assert hd.result_from_bytes(h_outs[k]) == refs[k % 2], f"e2e step {k}: result differs"
    # blocking: one hd_compute_u8 call per pair (the pack kernel reads the
    # pinned masks in place over the host link), and the same with explicit
    # host-to-device copies instead of in-place reads
    for w in range(max(1, args.warmup)):
        assert ctx.compute(*hpairs[w % 2], "se6") == refs[w % 2]
    blk_t = []
    for k in range(args.steps):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        r = ctx.compute(*hpairs[k % 2], "se6")
        blk_t.append((time.perf_counter() - t1) * 1000.0)
        assert r == refs[k % 2]
    blocking_e2e_ms = sum(blk_t) / len(blk_t)
    staged_ms = None
    with hd.Context(local, zero_copy=False) as sctx:
        assert sctx.compute(*hpairs[0], "se6") == refs[0]
        st_t = []
        for k in range(args.steps):
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            sctx.compute(*hpairs[k % 2], "se6")
            st_t.append((time.perf_counter() - t1) * 1000.0)
        staged_ms = sum(st_t) / len(st_t)
    if dist:
        t = torch.tensor([e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())

    # ---- phases of the launches the value path times --------------------------
    # the pipelined entry packs on a few SMs and dilates on the rest: CUDA
    # events on those streams around each kernel (the last of three
    # back-to-back calls: no packing runs beside its dilation, the previous
    # pair's dilation may, on the other SM group; over the four sequences the
    # last pair alternates between the two pairs)
    split_ph = []
    for k in range(4):
        for j in range(3):
            x, y = pairs[(k + j) % 2]
            tctx.compute_pipelined(x, y, "se6", out=outs[j])
        tctx.flush()
        torch.cuda.synchronize()
        tm = tctx.last_timings()
        if tm["iterations"] == -1:  # the split path ran
            split_ph.append(tm)
    # ---- roofline of the dominant kernel -------------------------------------
    # algorithmic bytes of the dilation (mean of the two pairs, like the times)
    tiles, bricks = 0, 0
    for x, y in pairs:
        res, tab, tba, br = ctx.profile(x, y, "se6")
        tiles += int(sum(int(v) for v in tab[1: res["hd_ab"] + 1]) + sum(int(v) for v in tba[1: res["hd_ba"] + 1]))
        bricks += br
    tiles /= 2
    bricks //= 2
    b_iter = 3 * 4096 * tiles
    b_pack = 2 * N + 2 * (N // 8)
    pk = statistics.mean(p["pack_ms"] for p in phases)
    su = statistics.mean(p["setup_ms"] for p in phases)
    so = statistics.mean(p["solve_ms"] for p in phases)
    peak, peak_kind = _peaks()
    share = {"pack": pk, "setup": su, "solve": so}
    dom = max(share, key=share.get)
    if dom == "solve":
        achieved = b_iter / (so * 1e-3) / 1e9
        alg = b_iter
    elif dom == "pack":
        achieved = b_pack / (pk * 1e-3) / 1e9
        alg = b_pack
    else:
        achieved = None
        alg = None
    kname = {"solve": "solve_tb_kernel" if phases[-1]["kernel"] == 2 else "solve_kernel",
             "pack": "pack_kernel", "setup": "setup_kernel"}[dom]
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            traffic = json.load(f).get("c2_512x512x256_se6", {}).get(kname)
    except Exception:
        traffic = None
    # the value path's dilation runs on the split SMs when the pipelined
    # entry split them: its solve time is what the frontier bytes are
    # divided by; the blocking entry's whole-GPU launch is reported beside it
    value_launch = None
    so_whole = so
    if split_ph and dom == "solve":
        so_split = statistics.mean(p["solve_ms"] for p in split_ph)
        value_launch = {
            "launch": f"solve_tb_kernel on the dilation SMs of the pipelined entry ({split_ph[0]['grid_ctas']} CTAs)",
            "solve_ms": round(so_split, 4), "pack_ms": round(statistics.mean(p["pack_ms"] for p in split_ph), 4),
            "setup_ms": round(statistics.mean(p["setup_ms"] for p in split_ph), 4),
            "achieved": round(b_iter / (so_split * 1e-3) / 1e9, 1)}
        value_launch["frac"] = round(value_launch["achieved"] / peak, 4)
        parts = split_ph[0].get("dilation_partitions", 1)
        value_launch["dilation_partitions"] = parts
        if parts > 1:
            # consecutive pairs dilate side by side on several SM groups: per
            # launch the time is longer, per pair the pipeline moves the
            # frontier bytes at the value leg's rate
            value_launch["launch"] += f", {parts} such launches in flight on disjoint SM groups"
            value_launch["pipeline"] = {
                "what": "frontier bytes of the value leg's pairs per second of its timed region",
                "achieved": round(b_iter * value / 1e9, 1), "frac": round(b_iter * value / 1e9 / peak, 4)}
        achieved = value_launch["achieved"]
        so = so_split
    roofline = {
        "bound": "hbm", "kernel": kname + {"solve": " (persistent frontier dilation)", "pack": " (uint8 -> bits)",
                                           "setup": " (crop + first queue)"}[dom],
        "achieved": round(achieved, 1) if achieved else None, "peak": peak, "unit": "GB/s",
        "frac": round(achieved / peak, 4) if achieved else None, "peak_source": f"{peak_kind} MEASURED_PEAKS hbm_gbs",
        "traffic": traffic, "algorithmic_bytes": alg,
        "phase_ms": {k: round(v, 4) for k, v in share.items()},
        "pack": {"bytes": b_pack, "ms": round(pk, 4), "gbs": round(b_pack / (pk * 1e-3) / 1e9, 1)},
        "solve": {"bytes": b_iter, "ms": round(so, 4), "gbs": round(b_iter / (so * 1e-3) / 1e9, 1),
                  "frontier_tiles": tiles, "bricks_processed": bricks},
    }
    if value_launch:
        roofline["traffic_source"] = ("ncu capture of the same kernel on every SM (bench.py --case c2): ncu cannot "
                                      "profile kernels launched in a green context")
        roofline["value_launch"] = value_launch
        roofline["whole_gpu_launch"] = {
            "launch": f"solve_tb_kernel of the blocking entry on every SM ({phases[-1]['grid_ctas']} CTAs)",
            "solve_ms": round(so_whole, 4), "achieved": round(b_iter / (so_whole * 1e-3) / 1e9, 1),
            "frac": round(b_iter / (so_whole * 1e-3) / 1e9 / peak, 4)}
    gvox = (refs[0]["hd"] + refs[1]["hd"]) / 2 * 2 * N / (step_ms * 1e-3) / 1e9

    out = {
        "metric": "mask-pairs/sec", "value": round(value, 3), "unit": "pairs/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32 (bit-packed binary masks, integer dilation counts)",
        "data": "synthetic seeded masks (reference data not available)",
        "config": {"workload": WORKLOAD, "W": W_, "H": H_, "D": D_, "element": "se6",
                   "l2": "inputs larger than L2: two distinct pairs alternate (2 x 134 MB of masks)",
                   "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
                   "kernel": "temporally blocked" if phases[-1]["kernel"] == 2 else "one step per barrier",
                   "steps_per_barrier": phases[-1]["steps_per_barrier"],
                   "brick_words_rows_planes": [phases[-1]["brick_x_words"], phases[-1]["brick_rows"],
                                               phases[-1]["brick_z"]], "grid_ctas": phases[-1]["grid_ctas"]},
        "hd": [refs[0]["hd"], refs[1]["hd"]], "avg_hd": [refs[0]["avg_hd"], refs[1]["avg_hd"]],
        "parity": "both pairs equal the oracle's stored results on every field (tests/golden/configs.json); "
                  "every timed result equals them",
        "barrier_iterations": [phases[0]["iterations"], phases[1]["iterations"]],
        "gvoxel_iter_per_s": round(gvox, 2),
        "e2e": {"value": round(ws * 1000.0 / e2e_ms, 3), "unit": "pairs/s", "ms_per_step": round(e2e_ms, 4),
                "h2d_bytes_per_step": 2 * N, "d2h_bytes_per_step": rbytes,
                "path": "hd_compute_u8_async: pinned host masks copied by DMA while the previous pair computes, "
                        "result read back to host each step; wall clock over the K steps",
                "blocking_ms_per_step": round(blocking_e2e_ms, 4),
                "blocking_path": "hd_compute_u8, one call per pair, masks read in place over the host link",
                "staged_copy_ms_per_step": round(staged_ms, 4)},
        "gpu_launches": 3 * args.steps,  # per pair: pack, set-up, persistent dilation (decodes the result too)
        "value_path": "hd_compute_u8_device_pipelined x K, hd_pipeline_flush: packing and set-up on 56 SMs, "
                      "consecutive pairs dilating side by side on three groups of 32 (green contexts, six "
                      "workspaces in turn)",
        "async_serial": {"path": "hd_compute_u8_device_async x K (each pair after the previous one)",
                         "ms_per_step": round(serial_ms, 4), "pairs_per_s": round(1000.0 / serial_ms, 1)},
        "blocking_call": {"path": "hd_compute_u8_device (returns the result to the host each call)",
                          "ms_per_step": round(statistics.mean(blocking), 4),
                          "pairs_per_s": round(1000.0 / statistics.mean(blocking), 1)},
        "roofline": roofline, "clocks": clk, "wall_s_timed_region": round(wall, 3),
    }

    if ws > 1 and not args.no_extras:
        # every rank: the 256-pair ragged batch split over the ranks
        out["sharded_batch"] = bench_sharded_batch(ctx, args, ws, rank, dist)
    if rank == 0 and ws == 1 and not args.no_extras:
        out["drop_in_default_element"] = bench_se18(ctx, pairs, seed)
        out["batched"] = bench_batched(ctx, args)
        out["worst_case"] = bench_worst_case(ctx, tctx, dev)
        out["serving"] = bench_serving(ctx, args)
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(a.cpu().numpy(), b.cpu().numpy(), refs[0])
    tctx.close()
    ctx.close()
    if dist:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out), flush=True)


_FIXTURE_KEYS = ("hd", "hd_ab", "hd_ba", "hd_robust", "sum_ab", "sum_ba", "n_a", "n_b", "n_a_not_b", "n_b_not_a",
                 "status", "avg_hd")
_FIXTURES = None


def _check_fixture(r, cfg, name, se, what):
    """r against the oracle's stored result for the same masks
    (tests/golden/configs.json, written by tests/golden/make_config_golden.py):
    every integer field identical and the same avg_hd double.  Entries the
    file does not hold (another seed under torchrun) are skipped."""
    global _FIXTURES
    if _FIXTURES is None:
        with open(os.path.join(ROOT, "tests", "golden", "configs.json")) as f:
            _FIXTURES = json.load(f)["configs"]
    o = _FIXTURES.get(cfg, {}).get(name, {}).get(se)
    if o is None:
        return False
    bad = [k for k in _FIXTURE_KEYS if r[k] != o[k] and not (k == "avg_hd" and o["status"] != 0)]
    assert not bad, f"{what}: fields {bad} differ from the oracle ({r} vs {o})"
    return True


def bench_batched(ctx, args):
    """256 ragged pairs: one persistent launch vs one call per pair (own
    contexts sharing one tuning table: the timed calls uninstrumented, the
    phase times from an instrumented one)."""
    import torch

    import housdorffhdf5cmake_gb300 as hd
    from housdorffhdf5cmake_gb300 import synth
    specs = synth.batch_ragged_specs(77, n=256)
    pairs = [synth.pair_from_spec(s, "cuda") for s in specs]
    voxels = sum(s.shape[0] * s.shape[1] * s.shape[2] for s in specs)
    # the autotuner times every compiled brick shape / steps per barrier /
    # grid size on these pairs (checking they agree) and keeps the fastest
    # for this workload class; the timed batches below use its choice
    tdir = tempfile.mkdtemp(prefix="hd_tune_")
    tpath = os.path.join(tdir, "tuning.json")
    ctx = hd.Context(ctx.device, tuning_table=tpath)
    report = ctx.autotune(pairs, "se6", repeats=3)
    tuned = [ln for ln in report.splitlines() if ln.startswith("best")]
    # phase times from an instrumented context with the same tuning table
    tctx = hd.Context(ctx.device, tuning_table=tpath, record_timings=True)
    batch = ctx.batch(pairs, "se6")
    plain = [ctx.compute(a, b, "se6") for a, b in pairs]
    # every result field except `iterations` (the shared loop's length in a batch)
    keys = ("hd", "hd_ab", "hd_ba", "hd_robust", "sum_ab", "sum_ba", "n_a", "n_b", "n_a_not_b", "n_b_not_a",
            "status")
    exact = all(x[k] == y[k] for x, y in zip(batch, plain) for k in keys)
    # every pair of the batch against the oracle's result for its masks
    oracle_checked = sum(_check_fixture(r, "c4", f"pair{i:03d}", "se6", f"batch pair {i}") for i, r in enumerate(batch))
    stream = torch.cuda.current_stream()

    def timed(fn, reps):
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    reps = max(3, min(args.steps, 5))
    # the batch call as a loop over the same buffers makes it: descriptors
    # prepared once, results as numpy columns; the one-shot call (fresh
    # descriptors, a dict per pair) beside it
    prep = ctx.prepare_batch(pairs, "se6")
    cols = prep.run(columns=True)
    exact = exact and all(int(cols[k][i]) == batch[i][k] for i in range(len(batch)) for k in keys)
    t_batch = timed(lambda: prep.run(columns=True), reps)
    tb = tctx.batch(pairs, "se6")
    assert all(x[k] == y[k] for x, y in zip(tb, batch) for k in keys), "instrumented batch differs"
    bt = tctx.last_timings()
    t_batch_dicts = timed(lambda: ctx.batch(pairs, "se6"), reps)
    t_plain = timed(lambda: [ctx.compute(a, b, "se6") for a, b in pairs], reps)
    # device time alone (CUDA events around the kernels of each call)
    dev_plain = 0.0
    for a, b in pairs:
        tctx.compute(a, b, "se6")
        dev_plain += tctx.last_timings()["total_ms"]
    gvox = sum(max(0, r["hd"]) * 2 * (s.shape[0] * s.shape[1] * s.shape[2]) for r, s in zip(batch, specs))
    # roofline of the batch's dilation launch: the frontier bytes of every
    # pair (32^3 tiles gaining voxels per step, counted by the instrumented
    # run) over the batch's solve time
    tiles = 0
    for (a, b), r in zip(pairs, batch):
        if r["status"] != 0:
            continue
        res, tab, tba, _ = ctx.profile(a, b, "se6")
        tiles += int(sum(int(v) for v in tab[1: res["hd_ab"] + 1]) + sum(int(v) for v in tba[1: res["hd_ba"] + 1]))
    b_iter = 3 * 4096 * tiles
    peak, peak_kind = _peaks()
    solve_gbs = b_iter / (bt["solve_ms"] * 1e-3) / 1e9
    out = {
        "workload": "256 ragged pairs, axes uniform in {64..384}, 5% edge pairs (empty / identical)",
        "pairs": len(pairs), "voxels": voxels,
        "batched_pairs_per_s": round(256 * 1000.0 / t_batch, 2), "batched_ms": round(t_batch, 3),
        "batched_path": "PreparedBatch.run(columns=True): one hd_batch_compute over descriptors built once",
        "batched_one_shot_ms": round(t_batch_dicts, 3),
        "batched_one_shot_path": "Context.batch: descriptors built and one result dict per pair, every call",
        "plain_pairs_per_s": round(256 * 1000.0 / t_plain, 2), "plain_ms": round(t_plain, 3),
        "speedup_batched_vs_plain": round(t_plain / t_batch, 2),
        "device_ms": {"batched": round(bt["total_ms"], 3), "plain_sum": round(dev_plain, 3),
                      "speedup": round(dev_plain / bt["total_ms"], 2)},
        "gvoxel_iter_per_s_batched": round(gvox / (t_batch * 1e-3) / 1e9, 2),
        "batched_phase_ms": {"pack": round(bt["pack_ms"], 3), "setup": round(bt["setup_ms"], 3),
                             "solve": round(bt["solve_ms"], 3), "barrier_iterations": bt["iterations"]},
        "pack_gbs_batched": round((2 * voxels + 2 * voxels / 8) / (bt["pack_ms"] * 1e-3) / 1e9, 1),
        "solve_roofline": {"bound": "hbm", "algorithmic_bytes": b_iter, "frontier_tiles": tiles,
                           "solve_ms": round(bt["solve_ms"], 4), "achieved": round(solve_gbs, 1), "peak": peak,
                           "unit": "GB/s", "frac": round(solve_gbs / peak, 4),
                           "peak_source": f"{peak_kind} MEASURED_PEAKS hbm_gbs"},
        "bit_exact_vs_plain": bool(exact), "pairs_checked_against_oracle": int(oracle_checked),
        "autotuned": tuned[0] if tuned else None,
        "shape": {"kernel": bt["kernel"], "steps_per_barrier": bt["steps_per_barrier"],
                  "brick_words_rows_planes": [bt["brick_x_words"], bt["brick_rows"], bt["brick_z"]],
                  "grid_ctas": bt["grid_ctas"]},
    }
    tctx.close()
    ctx.close()
    shutil.rmtree(tdir, ignore_errors=True)
    return out


def bench_se18(ctx, pairs, seed):
    """The headline pairs under the 18-neighbour element, the C++ drop-in's
    default (CHEBYSHEV 1): its domain is the bounding box of A u B with a
    one-voxel margin (shortest paths of that element may step out of the
    box), through the blocking device entry; each result checked against the
    oracle's."""
    import torch
    stream = torch.cuda.current_stream()
    ts, hds, checked = [], [], 0
    for i, (x, y) in enumerate(pairs):
        r = ctx.compute(x, y, "se18")
        checked += _check_fixture(r, "c2", f"pair{i}_seed{seed + i}", "se18", f"headline pair {i}, 18-neighbour element")
        hds.append(r["hd"])
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.compute(x, y, "se18")
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
    t = statistics.median(ts)
    return {"workload": "the two headline pairs, 18-neighbour element (forBench CHEBYSHEV 1)",
            "hd": hds, "ms_per_pair": round(t, 4), "pairs_per_s": round(1000.0 / t, 1),
            "path": "hd_compute_u8_device (blocking, result on the host)", "pairs_checked_against_oracle": int(checked)}


def bench_sharded_batch(ctx, args, ws, rank, dist):
    """Multi-GPU batches: the 256 ragged pairs split over the ranks
    largest-first (shard.plan_shards), each rank's share in one persistent
    launch (ctx.batch), the result records gathered on the host
    (shard.batch_sharded).  Time: barrier-bracketed, max over ranks."""
    import torch

    from housdorffhdf5cmake_gb300 import shard, synth
    specs = synth.batch_ragged_specs(77, n=256)
    costs = [s.shape[0] * s.shape[1] * s.shape[2] for s in specs]
    mine = shard.plan_shards(costs, ws)[rank]
    pairs = [None] * len(specs)
    for i in mine:  # each rank builds only its own share's masks
        pairs[i] = synth.pair_from_spec(specs[i], "cuda")
    torch.cuda.synchronize()
    run = lambda: shard.batch_sharded(pairs, lambda ps: ctx.batch(ps, "se6"), costs=costs)
    res = run()  # warm-up (and the check below)
    ts = []
    for _ in range(max(2, min(args.steps, 5))):
        dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        run()
        torch.cuda.synchronize()
        dist.barrier()
        ts.append(time.perf_counter() - t0)
    t = torch.tensor([statistics.median(ts)], device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    checked = sum(_check_fixture(r, "c4", f"pair{i:03d}", "se6", f"sharded batch pair {i}") for i, r in enumerate(res))
    return {"workload": "256 ragged pairs split over the ranks (largest-first), one batch launch per rank, "
                        "results gathered on the host",
            "ranks": ws, "ms": round(float(t.item()) * 1e3, 3),
            "pairs_per_s": round(len(specs) / float(t.item()), 1),
            "pairs_on_rank0": len(shard.plan_shards(costs, ws)[0]), "pairs_checked_against_oracle": int(checked)}


def bench_serving(ctx, args):
    """Serving: an open-loop Poisson stream of pairs through the continuous-
    batching server (hd_server_*), device-resident masks, 120 GB admission
    budget.  Pair sizes follow the serving distribution (log-normal volume
    around 256x256x160, aspect kept, capped at 512^3, 10% forced 512^3);
    requests cycle through a pool of distinct pairs.  For each offered rate:
    achieved pairs/s and p50 / p99 latency (submit -> result seen by the
    client).  The one-pair-at-a-time path is timed per pool pair and replayed
    as a FIFO single server on the same arrival times (its service times are
    deterministic), which gives its latencies at the same offered rates."""
    import threading

    import torch

    import housdorffhdf5cmake_gb300 as hd
    from housdorffhdf5cmake_gb300 import synth
    pool_n, n_req = 48, 400
    base = synth.serving_stream(4242, n=pool_n, rate_hz=0.0)
    pool = [synth.pair_for_request(r, "cuda") for r in base]
    torch.cuda.synchronize()
    want = [ctx.compute(a, b, "se6") for a, b in pool]
    for i, r in enumerate(want):
        _check_fixture(r, "c5", f"req{i:02d}", "se6", f"serving pool pair {i}")
    # one-pair-at-a-time service times (device-resident masks, result read back)
    svc = []
    for i, (a, b) in enumerate(pool):
        ts = []
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ctx.compute(a, b, "se6")
            ts.append(time.perf_counter() - t0)
        svc.append(min(ts))
    plain_rate = len(svc) / sum(svc)
    keys = ("hd", "hd_ab", "hd_ba", "sum_ab", "sum_ba", "n_a", "n_b", "status")

    def run(srv, rate):
        stream = synth.serving_stream(77 + int(rate), n=n_req, rate_hz=rate) if rate else None
        arr = [r.t_arrival for r in stream] if stream else [0.0] * n_req
        lat = [None] * n_req
        exact = [True]
        sub = {}  # ticket -> (request index, submit time)
        ticks0 = srv.stats()["ticks"]
        if True:
            def collect():
                # hd_server_wait_any: each finished request as soon as the
                # server completes it, in completion order
                for _ in range(n_req):
                    t, r = srv.wait_any(60000)
                    t_done = time.perf_counter()
                    while t not in sub:  # the submitter records the ticket right after submit returns
                        pass
                    i, t_sub = sub[t]
                    lat[i] = t_done - t_sub
                    w = want[i % pool_n]
                    if any(r[k] != w[k] for k in keys):
                        exact[0] = False
            th = threading.Thread(target=collect)
            th.start()
            t0 = time.perf_counter()
            lag = 0.0
            for i in range(n_req):
                # sleep until shortly before the arrival, then spin (the GIL
                # is handed over every 20 us, so the collector is not held up)
                gap = t0 + arr[i] - time.perf_counter()
                if gap > 3e-4:
                    time.sleep(gap - 2e-4)
                while time.perf_counter() - t0 < arr[i]:
                    pass
                t_sub = time.perf_counter()
                lag = max(lag, t_sub - t0 - arr[i])
                a, b = pool[i % pool_n]
                sub[srv.submit(a, b)] = (i, t_sub)
            th.join()
            t_end = time.perf_counter()
            st = srv.stats()
            st["ticks"] -= ticks0
        lat_ms = sorted(x * 1e3 for x in lat)
        # the one-pair-at-a-time path on the same arrivals: FIFO replay
        done, pl = 0.0, []
        for i in range(n_req):
            start = max(done, arr[i])
            done = start + svc[i % pool_n]
            pl.append((done - arr[i]) * 1e3)
        pl.sort()
        q = lambda v, f: round(v[min(len(v) - 1, int(f * len(v)))], 3)
        return {"offered_pairs_per_s": round(rate, 1) if rate else "burst",
                "achieved_pairs_per_s": round(n_req / (t_end - t0), 1),
                "p50_ms": q(lat_ms, 0.50), "p99_ms": q(lat_ms, 0.99),
                "plain_fifo_p50_ms": q(pl, 0.50), "plain_fifo_p99_ms": q(pl, 0.99),
                "max_submit_lag_ms": round(lag * 1e3, 3), "ticks": st["ticks"], "bit_exact": exact[0]}

    switch = sys.getswitchinterval()
    sys.setswitchinterval(2e-5)
    try:
        # one server for every rate, warmed up by a burst of the whole
        # stream (its memory pool then holds what the timed runs need)
        with hd.Server(ctx, hbm_budget_bytes=120 << 30) as srv:
            run(srv, 0.0)
            rows = [run(srv, f * plain_rate) for f in (0.5, 0.9, 1.5, 3.0)]
            rows.append(run(srv, 0.0))  # every request at t = 0: saturation throughput
    finally:
        sys.setswitchinterval(switch)
    return {"workload": "open-loop Poisson stream, sizes log-normal around 256x256x160 (cap 512^3, 10% 512^3), "
                        f"{n_req} requests per rate from a pool of {pool_n} distinct pairs, 6-neighbour element",
            "pool_voxels_mean": int(statistics.mean(s.shape[0] * s.shape[1] * s.shape[2] for s in base)),
            "plain_pairs_per_s": round(plain_rate, 1),
            "saturation_pairs_per_s": rows[-1]["achieved_pairs_per_s"],
            "saturation_vs_plain": round(rows[-1]["achieved_pairs_per_s"] / plain_rate, 2),
            "rates": rows}


def bench_worst_case(ctx, tctx, dev):
    """512^3, 8 small blobs vs 8 blobs >= 200 voxels away: long sparse frontier."""
    import torch

    from housdorffhdf5cmake_gb300 import synth
    a, b = synth.pair_far_blobs(5, (512, 512, 512), dev)
    ctx.compute(a, b, "se6")
    stream = torch.cuda.current_stream()
    ts = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = ctx.compute(a, b, "se6")
        e1.record(stream)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    t = statistics.median(ts)
    assert tctx.compute(a, b, "se6") == r
    tim = tctx.last_timings()
    checked = _check_fixture(r, "c3", "far_blobs_seed5", "se6", "512^3 far blobs")
    res, tab, tba, bricks = ctx.profile(a, b, "se6")
    nz = torch.nonzero(a | b)
    lo, hi = nz.min(0).values.tolist(), nz.max(0).values.tolist()  # (z, y, x)
    bxw, bz, by = tim["brick_x_words"], tim["brick_z"], tim["brick_rows"]
    wx = (hi[2] // 32) - (lo[2] // 32) + 1
    # profile() uses the one-step kernel with 4 x 8 x 8 bricks
    dom_bricks_1 = -(-wx // 4) * -(-(hi[1] - lo[1] + 1) // 8) * -(-(hi[0] - lo[0] + 1) // 8)
    iters = max(1, res["hd_ab"]) + max(1, res["hd_ba"])  # profile() runs the one-step kernel
    N = 512 ** 3
    # per dilation step: 32^3 tiles (of the 16^3 = 4096 of the volume) that
    # gained voxels, both directions; their algorithmic bytes over the solve
    n_tiles = (512 // 32) ** 3
    steps = max(res["hd_ab"], res["hd_ba"])
    per_step = [(int(tab[k]) if k <= res["hd_ab"] else 0) + (int(tba[k]) if k <= res["hd_ba"] else 0)
                for k in range(1, steps + 1)]
    frac = [x / (2 * n_tiles) for x in per_step]
    alg = 3 * 4096 * sum(per_step)
    return {
        "workload": "512^3, 8 balls r 3-6 vs 8 balls >= 200 voxels away, 6-neighbour element",
        "hd": r["hd"], "checked_against_oracle": bool(checked),
        "barrier_iterations": tim["iterations"], "steps_per_barrier": tim["steps_per_barrier"],
        "ms": round(t, 3), "ms_per_step": round(t / max(1, r["hd"]), 4),
        "pairs_per_s": round(1000.0 / t, 3),
        "gvoxel_iter_per_s": round(r["hd"] * 2 * N / (t * 1e-3) / 1e9, 2),
        "active_brick_fraction_mean": round(bricks / (dom_bricks_1 * iters), 4),
        "active_tile_fraction_per_step": {"every_25th": [round(f, 4) for f in frac[::25]],
                                          "mean": round(statistics.mean(frac), 4), "max": round(max(frac), 4)},
        "solve_algorithmic_gbs": round(alg / (tim["solve_ms"] * 1e-3) / 1e9, 1),
        "solve_ms": round(tim["solve_ms"], 3), "pack_ms": round(tim["pack_ms"], 3),
    }


def cpu_baseline(a_np, b_np, ref):
    """Serial restatement of the reference loop on the host (1 core)."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    o = O.forbench(a_np, b_np, "se6", nthreads=1)
    dt = time.perf_counter() - t0
    keys = ("hd", "hd_ab", "hd_ba", "sum_ab", "sum_ba", "n_a", "n_b", "n_a_not_b", "n_b_not_a", "status", "avg_hd")
    assert all(o[k] == ref[k] for k in keys), (o, ref)
    return {"value": round(1.0 / dt, 5), "unit": "pairs/s", "cores": 1, "kind": "port",
            "sample": f"the full headline pair ({W_}x{H_}x{D_}), one run, {dt:.1f} s, "
                      "oracle restatement of forBench/HausdorffDistance.cu:101-187 (serial scatter form)",
            "seconds": round(dt, 3)}


def bench_reference(args):
    """The reference algorithm on the host cores (oracle port, all threads)."""
    ws, rank, local = _dist_env()
    if rank != 0:
        return
    import numpy as np

    from housdorffhdf5cmake_gb300 import synth
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    # the same two pairs the GPU arm alternates
    pairs = [tuple(m.numpy() for m in synth.pair_shifted_union(1234 + i, (D_, H_, W_), "cpu")) for i in range(2)]
    for w in range(args.warmup):
        O.forbench(*pairs[w % 2], "se6", nthreads=threads)
    ts = []
    t_all = time.perf_counter()
    for k in range(args.steps):
        t0 = time.perf_counter()
        o = O.forbench(*pairs[k % 2], "se6", nthreads=threads)
        ts.append(time.perf_counter() - t0)
    t_all = time.perf_counter() - t_all
    step = sum(ts) / len(ts)
    v = 1.0 / step
    out = {
        "impl": "reference", "metric": "mask-pairs/sec", "value": round(v, 5), "unit": "pairs/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step * 1000, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8 (byte per voxel)",
        "data": "synthetic seeded masks (reference data not available)",
        "config": {"workload": WORKLOAD, "W": W_, "H": H_, "D": D_, "element": "se6"},
        "hd": o["hd"],
        "cpu_baseline": {"value": round(v, 5), "unit": "pairs/s", "cores": threads, "kind": "port",
                         "sample": "the full headline pair per step (the two pairs of the GPU arm in turn): oracle "
                                   "restatement of forBench/HausdorffDistance.cu:101-187, OpenMP scatter, all host threads"},
        "e2e": {"value": round(v, 5), "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(out), flush=True)


def run_case(args):
    """One workload, run a few times with nothing else around it, for
    profiler captures (no JSON line): c2 = the 512x512x256 pair (seed 1234),
    c3 = the 512^3 far-blobs pair, batch = the first --pairs pairs of the
    256-pair ragged batch in one launch."""
    import torch

    import housdorffhdf5cmake_gb300 as hd
    from housdorffhdf5cmake_gb300 import synth
    ctx = hd.Context(0, record_timings=True)
    if args.case == "batch":
        specs = synth.batch_ragged_specs(77, n=256)[: args.pairs]
        pairs = [synth.pair_from_spec(s, "cuda") for s in specs]
        run = lambda: ctx.batch(pairs, "se6")
    else:
        if args.case == "c2":
            a, b = synth.pair_shifted_union(1234, (D_, H_, W_), "cuda")
        else:
            a, b = synth.pair_far_blobs(5, (512, 512, 512), "cuda")
        run = lambda: ctx.compute(a, b, "se6")
    solves = []
    for _ in range(args.repeat):
        run()
        solves.append(ctx.last_timings()["solve_ms"])
    torch.cuda.synchronize()
    t = ctx.last_timings()
    t["solve_ms_median"] = statistics.median(solves)
    print(args.case, json.dumps(t), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-extras", action="store_true", help="skip the batched and worst-case sub-results")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--case", choices=["c2", "c3", "batch"], default=None,
                    help="run one workload --repeat times for a profiler capture (no JSON line)")
    ap.add_argument("--repeat", type=int, default=3)
    ap.add_argument("--pairs", type=int, default=64)
    args = ap.parse_args()
    if args.case:
        run_case(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        bench_reference(args)
    else:
        bench_ours(args)


if __name__ == "__main__":
    main()
