"""Multi-GPU mode of bench.py is replicas only: every rank relaxes its own
copy with no data exchange, the ranks meet at barriers around the timed
region and the time is the maximum over ranks.  These CPU tests run that
logic as two gloo ranks (no GPU): the rendezvous, the max-over-ranks
reduction, and the reference arm under torchrun, where ranks other than 0
exit at once."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": "2",
                       "RANK": str(rank), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import bench
    ws, r, local, dist = bench.dist_init()
    bench.barrier(dist)
    t = bench.max_over_ranks(1.5 + r, dist)
    bench.barrier(dist)
    res = {"ws": ws, "rank": r, "local": local, "max": t}
    if r != 0:
        # the reference arm: only rank 0 runs and prints
        class A:
            workload, steps, warmup = "disc_hole_2d", 1, 0
        res["reference_arm"] = bench.run_reference(A(), ws, r, dist)
    dist.destroy_process_group()
    out.put(res)


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=120) for _ in procs], key=lambda d: d["rank"])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [d["ws"] for d in res] == [2, 2]
    assert [d["local"] for d in res] == [0, 1]
    assert all(d["max"] == 2.5 for d in res)
    assert res[1]["reference_arm"] is None
