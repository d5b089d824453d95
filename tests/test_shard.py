"""Batches split over ranks (host-side logic, CPU only).

The planner is checked directly; the split-compute-gather path runs as two
gloo ranks on 127.0.0.1, each computing its share with the oracle (standing in
for a GPU rank's ``ctx.batch``), and must return every pair's result, in input
order, equal to computing the whole batch in one process.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from housdorffhdf5cmake_gb300.shard import batch_sharded, pair_cost, plan_shards


def test_plan_is_a_partition_and_balanced():
    rng = np.random.default_rng(3)
    costs = [int(x) for x in rng.integers(1, 1000, size=57)]
    for ws in (1, 2, 3, 8):
        shards = plan_shards(costs, ws)
        flat = sorted(i for s in shards for i in s)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in s) for s in shards]
        # largest-first greedy: max load <= mean + largest item
        assert max(loads) <= sum(costs) / ws + max(costs)
        assert plan_shards(costs, ws) == shards  # deterministic


def test_plan_edge_cases():
    assert plan_shards([], 2) == [[], []]
    assert plan_shards([5], 3) == [[0], [], []]
    assert plan_shards([1, 1, 1, 1], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        plan_shards([1], 0)


def test_pair_cost_is_voxels():
    assert pair_cost(np.zeros((3, 4, 5), np.uint8)) == 60


def _pairs():
    rng = np.random.default_rng(11)
    out = []
    for i in range(9):
        shape = tuple(int(x) for x in rng.integers(4, 14, size=3))
        a = (rng.random(shape) < 0.1).astype(np.uint8)
        b = (rng.random(shape) < 0.1).astype(np.uint8)
        if i == 4:
            b[:] = 0  # one-sided empty
        out.append((a, b))
    return out


def _oracle_batch(pairs):
    from oracle import oracle as O
    return [O.forbench(a, b, "se6") for a, b in pairs]


def _same(xs, ys):
    """Result lists equal field by field (NaN average on empty pairs matches NaN)."""
    if len(xs) != len(ys):
        return False
    for x, y in zip(xs, ys):
        if x.keys() != y.keys():
            return False
        for k in x:
            if x[k] != y[k] and not (isinstance(x[k], float) and x[k] != x[k] and y[k] != y[k]):
                return False
    return True


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        calls = []

        def compute(part):
            calls.append(len(part))
            return _oracle_batch(part)

        res = batch_sharded(_pairs(), compute)
        q.put((rank, res, calls))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_gather_every_result_in_order(oracle):
    want = _oracle_batch(_pairs())
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    got.sort(key=lambda t: t[0])
    shards = plan_shards([pair_cost(a) for a, _ in _pairs()], 2)
    for rank, res, calls in got:
        assert _same(res, want)
        assert calls == [len(shards[rank])]  # each rank computed only its share


def test_without_process_group_runs_locally():
    pairs = _pairs()[:3]
    assert _same(batch_sharded(pairs, _oracle_batch), _oracle_batch(pairs))


def _library_shaped_batch(pairs):
    """A compute with the library's result records: the fields of hd_result
    (housdorffhdf5cmake_gb300._native.HdResult), filled from the oracle."""
    from housdorffhdf5cmake_gb300 import _native as N
    from oracle import oracle as O
    out = []
    for a, b in pairs:
        o = O.forbench(a, b, "se6")
        r = N.HdResult()
        for f, _ in N.HdResult._fields_:
            if f in o:
                setattr(r, f, o[f])
        out.append(r.as_dict())
    return out


def _rank_library_records(rank, ws, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        res = batch_sharded(_pairs(), _library_shaped_batch)
        q.put((rank, res))
    finally:
        dist.destroy_process_group()


def test_sharded_gather_of_library_records_world2():
    """batch_sharded over two gloo ranks with a compute that returns the
    library's result records (what ctx.batch returns): every pair's record,
    in input order, equal to the whole batch in one process."""
    want = _library_shaped_batch(_pairs())
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    procs = [ctx.Process(target=_rank_library_records, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        assert len(got[r]) == len(want)
        for x, y in zip(got[r], want):
            assert set(x) == set(y)
            assert all(x[k] == y[k] or (x[k] != x[k] and y[k] != y[k]) for k in x)
