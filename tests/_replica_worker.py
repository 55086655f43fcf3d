"""Child process body for the two-rank replica tests (gloo on CPU)."""
import os


def oracle_runner(fail_rank):
    def run(mine):
        import torch.distributed as dist
        from tests import _oracle
        if dist.get_rank() == fail_rank:
            raise RuntimeError("simulated worker failure")
        out = []
        for k, n, tag in mine:
            o = _oracle.proth_test(k, n)
            out.append({"tag": tag, "k": k, "n": n, "verdict": o["verdict"], "res64": o["res64"],
                        "rank": dist.get_rank()})
        return out
    return run


def main(rank, world, port, cands, fail_rank, out_path):
    import json
    from datetime import timedelta

    import torch.distributed as dist

    from prothlogic_gb300 import replicas

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=timedelta(seconds=60))
    try:
        res = replicas.run_sharded(cands, oracle_runner(fail_rank))
        err = None
    except replicas.ReplicaError as exc:
        res, err = None, str(exc)
    if rank == 0:
        with open(out_path, "w") as f:
            json.dump({"results": res, "error": err}, f)
    dist.destroy_process_group()
