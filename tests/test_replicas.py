"""Multi-GPU runs are replicas (independent chains per rank, no collective on
the data path): the host-side logic of bench.py for N > 1 -- the job time is
the slowest rank's, the value counts every rank's steps, the reference arm
runs on rank 0 only -- exercised with two gloo ranks on the CPU."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _rank(rank, port, q):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2")
    dist.init_process_group("gloo", rank=rank, world_size=2)
    t = [1.5, 2.5][rank]
    t_all = bench.max_over_ranks(t, dist, "cpu")
    value = bench.job_value(100, 2, t_all)

    class A:
        steps, warmup, precision = 3, 3, "mixed"
    ref = bench.run_reference(A, 2, rank) if rank == 1 else "skipped"
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, t_all, value, ref))


def test_two_gloo_ranks():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t_all, value, ref in out:
        assert t_all == 2.5                      # the slowest rank's time
        assert value == pytest.approx(100 * 2 / 2.5)
    assert out[1][3] is None                     # the reference arm: rank 0 alone


def test_single_rank_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(1.25, None, "cpu") == 1.25
    assert bench.job_value(10, 1, 2.0) == 5.0
