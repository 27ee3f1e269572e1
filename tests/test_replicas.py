"""Multi-GPU is replicas only: every rank runs the whole workload and the job's time is the slowest rank's.
The rank reduction of bench.py is checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    v = bench.max_over_ranks(10.0 + 3.0 * rank, world)
    one = bench.max_over_ranks(7.0, 1)  # a single rank needs no process group
    out.put((rank, v, one))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    ps = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [13.0, 13.0]
    assert [r[2] for r in res] == [7.0, 7.0]
