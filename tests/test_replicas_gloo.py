"""CPU, two ranks over gloo: the multi-GPU path of bench.py is replicas only
(no data-path collective); its host logic -- the barrier, the max over ranks
of the timed seconds, the whole-job rate, and the reference arm's ranks other
than 0 exiting without work -- runs here on 127.0.0.1 without a GPU."""
import os
import socket
import sys

import pytest

from conftest import ROOT


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        local_s = 1.0 + rank  # rank 1 is the slow replica
        slowest = bench.max_over_ranks(dist, local_s, "cpu")
        rate = bench.whole_job_rate(world, 1000, slowest)
        # the reference arm: ranks other than 0 print nothing and return 0
        os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
        ref_rc = bench.run_reference(type("A", (), {"steps": 1, "warmup": 0, "gpus": world})()) \
            if rank != 0 else 0
        q.put((rank, slowest, rate, ref_rc))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, slowest, rate, ref_rc in got:
        assert slowest == 2.0                    # both ranks see the slowest replica's time
        assert rate == pytest.approx(2 * 1000 / 2.0)
        assert ref_rc == 0


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(None, 3.5, "cpu") == 3.5
    assert bench.whole_job_rate(1, 10, 2.0) == 5.0
