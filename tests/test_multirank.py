"""The multi-rank path of bench.py on CPU ranks (gloo, world size 2): each rank factors its
own batch (weak scaling, no collective on the data path), the step time is the maximum over
ranks, and the job's throughput counts every rank's batch.  The GPU side of each rank is the
single-GPU path tested elsewhere; only the host logic around it runs here."""
import multiprocessing as mp
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    import bench
    from genericschur_gb300.workloads import batched_real
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, _ = bench.dist_env()
        packed, ns, offs, woffs = batched_real(count=64, seed=bench.rank_seed(r))
        ms = 10.0 + 5.0 * r  # a slower rank 1
        m = bench.reduce_max_ms(torch, ms, w, torch.device("cpu"))
        v = bench.job_throughput(w, len(ns), m)
        q.put((r, w, len(ns), float(packed.sum()), m, v))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_shard_and_take_the_max():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    out.sort()
    (r0, w0, c0, s0, m0, v0), (r1, w1, c1, s1, m1, v1) = out
    assert (r0, r1) == (0, 1) and w0 == w1 == 2
    assert c0 == c1 == 64 and s0 != s1  # same size law, different batches
    assert m0 == m1 == 15.0            # the slower rank's step
    assert v0 == v1 == pytest.approx(2 * 64 / 0.015)


def test_single_rank_is_unchanged():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_max_ms(None, 12.5, 1, None) == 12.5
    assert bench.job_throughput(1, 100, 50.0) == pytest.approx(2000.0)
    assert bench.rank_seed(0) == bench.SEED


def test_reference_arm_other_ranks_exit_quietly():
    """Under torchrun only rank 0 times the CPU reference and prints its line; the other
    ranks return at once with exit status 0."""
    import subprocess
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""
