"""The replica layer of the benchmark with two ranks on CPU (gloo): every
rank gets its own circuit seed, only rank 0 leads, barriers hold, and the
job's throughput is all ranks' units over the slowest rank's time."""
import multiprocessing as mp
import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    from qsl_gb300.replicas import Replicas
    rep = Replicas("gloo")
    rep.barrier()
    units, seconds = 100.0 * (rank + 1), 2.0 + rank     # rank 1 is the slowest
    out.put((rank, rep.leader, rep.seed(7), rep.max(seconds), rep.sum(units),
             rep.throughput(units, seconds)))
    rep.close()


def test_two_replicas_on_gloo():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, lead0, seed0, mx0, sm0, tp0), (r1, lead1, seed1, mx1, sm1, tp1) = res
    assert (lead0, lead1) == (True, False)
    assert (seed0, seed1) == (7, 8)
    assert mx0 == mx1 == 3.0 and sm0 == sm1 == 300.0
    assert tp0 == tp1 == pytest.approx(100.0)


def test_single_rank_makes_no_collective(monkeypatch):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    from qsl_gb300.replicas import Replicas
    rep = Replicas("gloo")
    assert rep.world == 1 and rep.leader and rep.dist is None
    assert rep.throughput(50.0, 2.0) == 25.0
    rep.close()
