"""The replica coordination of bench.py under torchrun, on CPU: two gloo
ranks meet at a barrier, agree on the slowest rank's time, and count the
whole job's work."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    from zpic_gb300.replicas import Replicas

    r = Replicas(backend="gloo")
    r.barrier()
    t = 1.0 + rank          # rank 1 is the slow one
    out[rank] = (r.allmax(t), r.throughput(100.0, t), r.world)
    r.close()


def test_two_gloo_replicas():
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        tmax, thr, w = res[rank]
        assert w == 2
        assert tmax == 2.0
        assert thr == 100.0 * 2 / 2.0


def test_single_process_needs_no_group():
    from zpic_gb300.replicas import Replicas

    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    r = Replicas()
    assert r.world == 1 and r.dist is None
    assert r.allmax(3.5) == 3.5
    assert r.throughput(10.0, 2.0) == 5.0
    r.close()
