"""The multi-GPU form of bench.py is independent replicas (no exchange on the data path):
its only collective is the max-over-ranks of the step times.  Checked here with two gloo
ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    t = bench.max_over_ranks([0.010 + 0.005 * rank, 0.020 - 0.005 * rank], world)
    out[rank] = (t, bench.replica_rate(1000, t[0], world))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_max_and_rate():
    mp = pytest.importorskip('torch.multiprocessing')
    ctx = mp.get_context('spawn')
    port = _free_port()
    with ctx.Manager() as man:
        out = man.dict()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        for r in range(2):
            t, rate = out[r]
            assert t == pytest.approx([0.015, 0.020])
            assert rate == pytest.approx(2 * 1000 / 0.015)
