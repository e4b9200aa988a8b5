"""The multi-GPU path of bench.py is replicas only (one Hamiltonian per GPU, no
collective in the data path); its one exchange is the max over ranks of the
timed region.  Two gloo ranks on the CPU check that every rank sees the
slowest replica's time and that the whole-job rate counts every replica."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        m = bench.max_over_ranks(times[rank], "cpu")
        out.put((rank, m, bench.whole_job_rate(100, world, m)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    times = [12.5, 20.0]  # ms of each replica's timed region
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, m, rate in res:
        assert m == 20.0
        assert rate == pytest.approx(2 * 100 / 0.020)


def test_single_process_is_its_own_max():
    import bench
    assert bench.max_over_ranks(3.0, "cpu") == 3.0
    assert bench.whole_job_rate(10, 1, 5.0) == pytest.approx(2000.0)
