"""The N > 1 path of bench.py on the host: two ranks over gloo, each with
its own replica and its own timing; barriers, the maximum over ranks and the
whole-job throughput (world x units / slowest time), as the GPU run does
them over NCCL."""
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


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    reps = bench.Replicas("gloo", "cpu")
    try:
        reps.barrier()
        seconds = 1.0 + rank          # rank 1 is the slowest
        units = 100.0
        value = reps.whole_job(units, seconds)
        top = reps.max(10.0 * (rank + 1))
        reps.barrier()
        out.put((rank, reps.world, value, top))
    finally:
        reps.close()


def test_replicas_two_ranks_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, out))
             for r in range(world)]
    for p in procs:
        p.start()
    res = [out.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, w, value, top in res:
        assert w == world
        assert value == pytest.approx(world * 100.0 / 2.0)
        assert top == 20.0


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK")
           if k in os.environ}
    try:
        reps = bench.Replicas("gloo", "cpu")
        assert reps.world == 1 and reps.rank == 0
        assert reps.max(3.5) == 3.5
        assert reps.whole_job(10.0, 2.0) == 5.0
        reps.barrier()
        reps.close()
    finally:
        os.environ.update(env)
