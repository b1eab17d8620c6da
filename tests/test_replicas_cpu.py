"""The multi-GPU path is replicas only: each rank searches its own copy of
the queries on its own copy of the index, and the ranks exchange only their
timings.  Checked here with two gloo processes on the CPU: the job's time is
the slowest rank's on every rank, and the rate counts every rank's queries."""
import os

import pytest


def _rank(rank, world, port, times, out):
    import torch.distributed as dist
    from song_gb300 import replicas as R
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    slow = R.max_over_ranks(times[rank], dist, "cpu")
    out.put((rank, slow, R.whole_job_rate(10000, 3, world, slow)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    import socket

    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    times = [1.5, 2.0]
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.0, 2.0]
    assert all(r[2] == pytest.approx(2 * 10000 * 3 / 2.0) for r in res)


def test_single_process_needs_no_group():
    from song_gb300 import replicas as R
    assert R.max_over_ranks(1.25) == 1.25
    assert R.whole_job_rate(100, 2, 1, 0.5) == 400.0
