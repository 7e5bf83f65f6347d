"""The N > 1 path of bench.py on CPU: two gloo ranks, each timing its own
replica; the reported rate is all ranks' units over the slowest rank's time."""

import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, seconds, out):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    from multiphase_flow_codes_gb300.replicas import Replicas
    rep = Replicas("gloo")
    rep.barrier()
    rate, slowest = rep.rate(1000.0, seconds[rank])
    out[rank] = (rate, slowest, rep.leader, rep.world)
    rep.close()


def test_two_ranks_rate_uses_slowest_rank():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        port = _free_port()
        seconds = [1.0, 4.0]
        procs = [ctx.Process(target=_worker, args=(r, 2, port, seconds, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(2):
        rate, slowest, leader, world = res[r]
        assert world == 2 and slowest == 4.0
        assert rate == pytest.approx(2 * 1000.0 / 4.0)
        assert leader == (r == 0)


def test_single_rank_without_process_group(monkeypatch):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    from multiphase_flow_codes_gb300.replicas import Replicas
    rep = Replicas("gloo")
    assert rep.world == 1 and rep.leader and rep.dist is None
    assert rep.rate(10.0, 2.0) == (5.0, 2.0)
    rep.close()
