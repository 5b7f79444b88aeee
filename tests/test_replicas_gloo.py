"""Multi-GPU path of bench.py (replicas only): the timing reduction and the
whole-job throughput, run as world_size 2 gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import torch.distributed as tdist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r "took" 1.0 + r seconds: the job time is the slowest rank's
    t = bench.reduce_max(1.0 + rank, "cpu")
    v = bench.replica_value(1000, world, t)
    tdist.barrier()
    tdist.destroy_process_group()
    out.put((rank, t, v))


def test_reduce_max_and_replica_value_two_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, v in res:
        assert t == 2.0
        assert v == 2 * 1000 / 2.0
