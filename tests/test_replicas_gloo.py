"""The multi-GPU path is replicas only: each rank steps its own batch and the
ranks meet once, to combine the timing.  Two gloo ranks on the CPU check that
combination (slowest rank's times, sum of the ranks' terms)."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    res = bench.combine_ranks(10.0 + rank, 1.0 + 0.5 * rank, 100 * (rank + 1), "cpu")
    dist.destroy_process_group()
    out.put((rank, res))


def test_two_gloo_ranks_combine_times_and_terms():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        assert got[r] == (11.0, 1.5, 300)


def test_single_process_returns_its_own_figures():
    pytest.importorskip("torch")
    import bench
    assert bench.combine_ranks(3.0, 0.25, 42, "cpu") == (3.0, 0.25, 42)
