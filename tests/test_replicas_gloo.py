"""The N > 1 path of bench.py: world_size-2 gloo ranks on the CPU (no GPU):
barrier, max-over-ranks timing and whole-job throughput."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, size, port, out):
    os.environ.update({'MASTER_ADDR': '127.0.0.1', 'MASTER_PORT': str(port),
                       'WORLD_SIZE': str(size), 'RANK': str(rank), 'LOCAL_RANK': str(rank)})
    from qgate_gb300 import replicas
    replicas.init()
    replicas.barrier()
    value, t = replicas.aggregate_throughput(100.0, 1.0 + rank)  # rank 1 is slower
    out.put((rank, value, t))
    replicas.finish()


def test_two_gloo_ranks_take_the_slowest_time():
    mp = pytest.importorskip('torch.multiprocessing')
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, t in res:
        assert t == 2.0
        assert value == 100.0 * 2 / 2.0


def test_single_rank_defaults():
    from qgate_gb300 import replicas
    for k in ('WORLD_SIZE', 'RANK', 'LOCAL_RANK'):
        os.environ.pop(k, None)
    assert replicas.world() == (1, 0, 0)
    assert replicas.aggregate_throughput(10.0, 2.0) == (5.0, 2.0)
