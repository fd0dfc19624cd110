"""The N > 1 path of bench.py on CPU ranks (gloo, world size 2): replicas
report the slowest rank's time, and the reference arm prints from rank 0
only.  (One GPU per box in this build, so the GPU side of the replicas runs
in the driver's scaling runs, not here.)"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out.put((rank, bench.reduce_max(10.0 * (rank + 1), dist)))
    finally:
        dist.destroy_process_group()


def test_reduce_max_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == {0: 20.0, 1: 20.0}


def test_reference_arm_silent_on_other_ranks(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        steps, warmup, gpus = 1, 0, 2
    assert bench.run_reference(A(), rank=1) == 0
    assert capsys.readouterr().out == ""
