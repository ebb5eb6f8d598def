"""The bench's replicas-only multi-GPU path on CPU: world_size-2 gloo ranks
(torch.distributed, 127.0.0.1).  Each rank runs its own replica set; the only
collective is the timing max and the unit sum over ranks (bench.reduce_max_sum),
and rank 0 alone prints."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    w, r, local = bench.dist_env()
    assert (w, r, local) == (world, rank, rank)
    d = bench.dist_init(w, "gloo")
    t, units = bench.reduce_max_sum(d, 1.0 + rank, 1000.0 * (rank + 1))
    out.put((rank, t, units))
    d.barrier()
    d.destroy_process_group()


def test_reduce_max_sum_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, t, units in res:
        assert t == 2.0 and units == 3000.0      # max of the times, sum of the units


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.dist_init(1, "gloo") is None
    assert bench.reduce_max_sum(None, 1.5, 10.0) == (1.5, 10.0)


def test_reference_arm_other_ranks_exit_quietly():
    """Under torchrun only rank 0 runs and prints the reference arm's line."""
    import subprocess
    import sys
    from conftest import ROOT
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "c1",
                        "--steps", "1", "--warmup", "3"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
