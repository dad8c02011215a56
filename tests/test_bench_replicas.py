"""bench.py's multi-GPU path: independent replicas, one process per GPU.

The timing helper (bench.Replicas) runs here as two gloo ranks on the CPU.
Every rank passes its own step time; all ranks must get the maximum, and the
barrier must hold the faster rank back until the slower one arrives."""
import os
import socket
import time

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "MASTER_ADDR": "127.0.0.1",
                       "MASTER_PORT": str(port), "LOCAL_RANK": str(rank)})
    import bench
    reps = bench.Replicas()
    time.sleep(0.3 * rank)           # rank 1 arrives late
    t0 = time.time()
    reps.barrier()
    waited = time.time() - t0
    ms = reps.max(1.5 + rank)        # per-rank step times 1.5 and 2.5
    out.put((rank, ms, waited, reps.world))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_replicas_max_and_barrier_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.5, 2.5]   # both ranks see the slowest replica's time
    assert res[0][2] >= 0.2                     # rank 0 waited for rank 1 at the barrier
    assert [r[3] for r in res] == [2, 2]


def test_replicas_single_process_is_identity():
    import bench
    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK") if k in os.environ}
    try:
        reps = bench.Replicas()
        assert reps.world == 1 and reps.max(3.25) == 3.25
        reps.barrier()
    finally:
        os.environ.update(env)
