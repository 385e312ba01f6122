"""The benchmark's N-GPU path (independent replicas, no data-path
collective) on the CPU: two gloo ranks with different step times combine
into the maximum step time and the work of both ranks."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, os.path.dirname(HERE))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms, value = bench.combine_replicas(10.0 + 5.0 * rank, 1.0e9, world)
        out.put((rank, ms, value))
    finally:
        dist.destroy_process_group()


def test_two_replicas_max_time_and_total_work():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value in res:
        assert ms == 15.0
        assert value == pytest.approx(2 * 1.0e9 / 15e-3)
