"""Replica sharding over ranks (one process per GPU): host logic on CPU, two
gloo ranks, the oracle standing in for each rank's engine."""
import json
import random
import socket

import pytest

from prothlogic_gb300 import replicas


def _cands(count, seed=7):
    rng = random.Random(seed)
    return [(2 * rng.randrange(1, 2000) + 1, rng.randrange(1500, 3000), tag) for tag in range(count)]


def test_shard_partitions_and_balances():
    cands = _cands(101)
    for world in (1, 2, 3, 8):
        parts = [replicas.shard(cands, world, r) for r in range(world)]
        tags = sorted(t for p in parts for _, _, t in p)
        assert tags == list(range(len(cands)))  # each candidate exactly once
        loads = [sum(replicas.cost(k, n) for k, n, _ in p) for p in parts]
        biggest = max(replicas.cost(k, n) for k, n, _ in cands)
        assert max(loads) - min(loads) <= biggest  # LPT bound
        assert parts == [replicas.shard(cands, world, r) for r in range(world)]  # deterministic
    with pytest.raises(ValueError):
        replicas.shard(cands, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run_two_ranks(tmp_path, cands, fail_rank):
    import torch.multiprocessing as mp
    from tests import _replica_worker
    out = tmp_path / "out.json"
    mp.start_processes(_replica_worker.main, args=(2, _free_port(), cands, fail_rank, str(out)), nprocs=2,
                       join=True, start_method="spawn")
    with open(out) as f:
        return json.load(f)


def test_two_gloo_ranks_gather_every_result(tmp_path, oracle):
    cands = _cands(12)
    got = _run_two_ranks(tmp_path, cands, fail_rank=-1)
    assert got["error"] is None
    res = got["results"]
    assert [r["tag"] for r in res] == list(range(len(cands)))
    assert {r["rank"] for r in res} == {0, 1}  # both ranks worked
    for (k, n, tag), r in zip(cands, res):
        o = oracle.proth_test(k, n)
        assert (r["k"], r["n"], r["verdict"], r["res64"]) == (k, n, o["verdict"], o["res64"])


def test_failed_rank_is_reported_not_waited_for(tmp_path, oracle):
    got = _run_two_ranks(tmp_path, _cands(6), fail_rank=1)
    assert got["results"] is None
    assert "rank 1" in got["error"] and "simulated worker failure" in got["error"]
