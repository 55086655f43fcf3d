"""Replica sharding: independent Proth candidates spread over one process per GPU.

A single candidate's squaring chain does not shard (every squaring is a full
transform of one residue, a few MB, that fits one GPU), so several GPUs run
independent replicas of the engine over disjoint sets of candidates, the way
the reference's dispatcher hands whole candidates to worker threads
(prothlogic4.2/dcore.cpp:125-188).  There is no collective on the data path:
the only exchange is the gathering of finished results to rank 0 at the end,
over the host process group (gloo).

    python -m torch.distributed.run --nproc-per-node 2 --master-addr 127.0.0.1 \\
        -m prothlogic_gb300.replicas --count 64 --n 65536
"""
import argparse
import heapq
import json
import math
import os
import time


def cost(k, n):
    """Relative cost of a full test: n squarings of an FFT of about n/16 points."""
    m = max(256.0, n / 16.0)
    return n * m * math.log2(m)


def shard(cands, world, rank):
    """Deterministic longest-processing-time split of `cands` [(k, n, tag)].

    Every candidate lands on exactly one rank; ranks get about equal total cost.
    Returns this rank's candidates in their original order."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad world/rank")
    order = sorted(range(len(cands)), key=lambda i: (-cost(cands[i][0], cands[i][1]), i))
    heap = [(0.0, r) for r in range(world)]
    owner = [0] * len(cands)
    for i in order:
        load, r = heapq.heappop(heap)
        owner[i] = r
        heapq.heappush(heap, (load + cost(cands[i][0], cands[i][1]), r))
    return [c for i, c in enumerate(cands) if owner[i] == rank]


class ReplicaError(RuntimeError):
    """A rank's runner failed; carries every failing rank's message."""


def run_sharded(cands, runner, pgd=None):
    """Run `runner(my_cands) -> [result dict with "tag"]` on this rank's shard.

    With a process group `pgd` (or the default group when torch.distributed is
    initialised) results are gathered to rank 0, which returns all of them
    sorted by tag; other ranks return None.  A rank whose runner raises reports
    the error instead of results, and rank 0 raises ReplicaError after the
    gather, so no rank waits forever on a failed peer."""
    import torch.distributed as dist

    world = dist.get_world_size(pgd) if dist.is_initialized() else 1
    rank = dist.get_rank(pgd) if dist.is_initialized() else 0
    mine = shard(cands, world, rank)
    try:
        out = {"rank": rank, "results": list(runner(mine)), "error": None}
    except Exception as exc:  # reported to rank 0, not raised here
        out = {"rank": rank, "results": [], "error": "%s: %s" % (type(exc).__name__, exc)}
    if world == 1:
        parts = [out]
    else:
        parts = [None] * world
        dist.all_gather_object(parts, out, group=pgd)
    if rank != 0:
        return None
    errors = ["rank %d: %s" % (p["rank"], p["error"]) for p in parts if p["error"]]
    if errors:
        raise ReplicaError("; ".join(errors))
    res = [r for p in parts for r in p["results"]]
    res.sort(key=lambda r: r["tag"])
    return res


def batch_runner(max_slots=1024):
    """Runner that tests a shard with the batched engine on this rank's GPU."""
    def run(mine):
        from . import Batch
        b = Batch(max_slots)
        for k, n, tag in mine:
            b.submit(k, n, tag)
        b.run(0)
        res = b.poll()
        b.close()
        return res
    return run


def main():
    import torch
    import torch.distributed as dist

    from . import set_device, workloads

    ap = argparse.ArgumentParser()
    ap.add_argument("--count", type=int, default=64)
    ap.add_argument("--n", type=int, default=65536)
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        dist.init_process_group("gloo")
    set_device(int(os.environ.get("LOCAL_RANK", "0")) % max(1, torch.cuda.device_count()))
    cands = [(k, args.n, i) for i, (k, _) in enumerate(workloads.uniform(args.count))]
    t0 = time.perf_counter()
    res = run_sharded(cands, batch_runner())
    if res is not None:
        wall = time.perf_counter() - t0
        print(json.dumps({"world": world, "tests": len(res), "wall_s": wall,
                          "tests_per_hour": len(res) / wall * 3600.0,
                          "primes": sum(1 for r in res if r["verdict"] == 1)}))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
