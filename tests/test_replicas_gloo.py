"""The multi-GPU path on the CPU: two gloo ranks.

Under torchrun the benches run replicas (glemur_gb300/replicas.py): each rank
its own relaxation, or its share of the batched cases, with only the timing
combined.  These tests run that host logic as two spawned processes over
gloo on 127.0.0.1: the job's time is the slowest rank's, the work is summed,
and the batched cases are split so that each runs on exactly one rank."""
import os
import socket

import pytest

from glemur_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist, r, w = replicas.init("gloo")
    try:
        ms = [12.5, 40.25][r]                   # this rank's timed region
        work = [1000.0, 3000.0][r]              # cell-RK-stages it did
        cases = replicas.shard(64, r, w)
        out[r] = dict(rank=r, ws=w, t=replicas.max_over_ranks(dist, ms),
                      work=replicas.sum_over_ranks(dist, work), cases=cases,
                      n_cases=replicas.sum_over_ranks(dist, len(cases)),
                      gathered=replicas.gather_lists(dist, [float(c) for c in cases]))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_combine_timing_and_split_cases():
    import torch.multiprocessing as mp
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
        res = [out[0], out[1]]
    for r, o in enumerate(res):
        assert o["rank"] == r and o["ws"] == 2
        assert o["t"] == 40.25                  # the slowest rank's time
        assert o["work"] == 4000.0              # work summed over ranks
        assert o["n_cases"] == 64
        assert o["gathered"] == [float(c) for c in res[0]["cases"] + res[1]["cases"]]
    a, b = set(res[0]["cases"]), set(res[1]["cases"])
    assert not a & b and a | b == set(range(64))
    assert len(a) == len(b) == 32


def test_single_process_needs_no_group(monkeypatch):
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    dist, rank, ws = replicas.init()
    assert dist is None and (rank, ws) == (0, 1)
    assert replicas.max_over_ranks(None, 3.5) == 3.5
    assert replicas.sum_over_ranks(None, 2.0) == 2.0
    assert replicas.gather_lists(None, [1, 2]) == [1, 2]
    assert replicas.shard(5, 0, 1) == [0, 1, 2, 3, 4]


def test_shard_is_a_partition_for_uneven_counts():
    for n in (0, 1, 7, 64, 65):
        for ws in (1, 2, 3, 8):
            parts = [replicas.shard(n, r, ws) for r in range(ws)]
            flat = sorted(i for p in parts for i in p)
            assert flat == list(range(n))
            assert max(map(len, parts)) - min(map(len, parts)) <= 1
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)
