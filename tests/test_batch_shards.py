"""The batching form split across ranks (qsl_gb300/batch_shards.py), on CPU.

The split is host logic: a cost-balanced partition of the instances, the
slicing of each rank's angles and uniforms, and the reassembly of the
gathered results in instance order.  A stand-in runner replaces the GPU
batch: its outputs depend on every angle and uniform of an instance, so a
misplaced slice or a misordered result changes them.  Two `gloo` ranks run
the gather the way two GPUs would."""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

from qsl_gb300 import batch_shards as bs

NSHOTS = 16


def fake_runner(ns, ls, angles, uniforms):
    """Per instance: probs (n, 2) = the angles summed over layers, shots =
    floor(u * 2^n); the same arithmetic whatever the batch around it."""
    probs, shots, at = [], [], 0
    nshots = np.asarray(uniforms).size // max(len(ns), 1)
    u = np.asarray(uniforms).reshape(len(ns), nshots)
    for k, (n, L) in enumerate(zip(ns, ls)):
        n, L = int(n), int(L)
        seg = angles[at:at + 2 * n * L].reshape(L, n, 2)
        at += 2 * n * L
        probs.append(seg.sum(axis=0))
        shots.append(np.floor(u[k] * (1 << n)).astype(np.uint64))
    return probs, np.stack(shots) if shots else np.empty((0, nshots), dtype=np.uint64)


def workload(seed, ninst=64):
    rng = np.random.default_rng(seed)
    ns = rng.integers(2, 21, ninst).astype(np.uint32)
    ls = rng.integers(1, 17, ninst).astype(np.uint32)
    angles = rng.uniform(0, 2 * np.pi, int(np.sum(2 * ns.astype(np.int64) * ls)))
    u = rng.random(ninst * NSHOTS)
    return ns, ls, angles, u


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_partition_is_complete_and_balanced(world):
    rng = np.random.default_rng(world)
    ns = rng.integers(10, 21, 4096)
    ls = rng.integers(4, 17, 4096)
    c = bs.instance_costs(ns, ls)
    parts = bs.partition_by_cost(c, world)
    allidx = np.sort(np.concatenate(parts))
    assert np.array_equal(allidx, np.arange(4096))
    loads = np.array([c[p].sum() for p in parts])
    assert loads.max() - loads.min() <= c.max()
    assert loads.max() <= 4 / 3 * c.sum() / world + c.max()
    again = bs.partition_by_cost(c, world)
    assert all(np.array_equal(a, b) for a, b in zip(parts, again))


def test_more_ranks_than_instances():
    parts = bs.partition_by_cost(np.array([5, 1], dtype=np.int64), 4)
    assert [p.tolist() for p in parts] == [[0], [1], [], []]


def test_select_and_assemble_round_trip():
    ns, ls, angles, u = workload(3)
    whole = fake_runner(ns, ls, angles, u)
    parts = bs.partition_by_cost(bs.instance_costs(ns, ls), 3)
    results = [fake_runner(*bs.select(ns, ls, angles, u, NSHOTS, p)) for p in parts]
    probs, shots = bs.assemble(ns, NSHOTS, parts, results)
    assert np.array_equal(shots, whole[1])
    assert all(np.array_equal(a, b) for a, b in zip(probs, whole[0]))


def test_assemble_rejects_missing_and_repeated_instances():
    ns, ls, angles, u = workload(4, ninst=6)
    parts = [np.array([0, 1, 2]), np.array([3, 4])]
    results = [fake_runner(*bs.select(ns, ls, angles, u, NSHOTS, p)) for p in parts]
    with pytest.raises(ValueError):
        bs.assemble(ns, NSHOTS, parts, results)
    parts = [np.array([0, 1, 2]), np.array([2, 3, 4, 5])]
    results = [fake_runner(*bs.select(ns, ls, angles, u, NSHOTS, p)) for p in parts]
    with pytest.raises(ValueError):
        bs.assemble(ns, NSHOTS, parts, results)


def test_select_checks_the_angle_count():
    ns, ls, angles, u = workload(5, ninst=4)
    with pytest.raises(ValueError):
        bs.select(ns, ls, angles[:-1], u, NSHOTS, np.array([0]))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    from qsl_gb300.replicas import Replicas
    rep = Replicas("gloo")
    ns, ls, angles, u = workload(11)
    probs, shots, mine = bs.run_sharded(rep, ns, ls, NSHOTS, angles, u, fake_runner)
    out.put((rank, [p.tolist() for p in probs], shots.tolist(), mine.tolist()))
    rep.close()


def test_two_ranks_gather_every_instance_in_order():
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
    ns, ls, angles, u = workload(11)
    whole = fake_runner(ns, ls, angles, u)
    (r0, probs0, shots0, mine0), (r1, probs1, shots1, mine1) = res
    assert sorted(mine0 + mine1) == list(range(len(ns))) and mine0 and mine1
    for probs, shots in ((probs0, shots0), (probs1, shots1)):
        assert np.array_equal(np.array(shots, dtype=np.uint64), whole[1])
        assert all(np.array_equal(np.array(a), b) for a, b in zip(probs, whole[0]))


class _StubBatch:
    """Stands in for qsl_gb300.Batch in the bench's sharded section."""

    def __init__(self, ns, ls, nshots, dtype):
        self.ns, self.ls = np.asarray(ns), np.asarray(ls)

    def autotune(self, angles, uniforms):
        return 1.0

    def run(self, angles, uniforms):
        return fake_runner(self.ns, self.ls, angles, uniforms)


class _PositionalStubBatch(_StubBatch):
    """A faulty batch: an instance's shots depend on its position within
    the batch, so a share run alone differs from the whole batch."""

    def run(self, angles, uniforms):
        probs, shots = fake_runner(self.ns, self.ls, angles, uniforms)
        return probs, shots + np.arange(len(self.ns), dtype=np.uint64)[:, None]


def _bench_rank_main(rank: int, world: int, port: int, out, stub=_StubBatch):
    import sys
    import types
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    from qsl_gb300.replicas import Replicas
    rep = Replicas("gloo")
    q = types.SimpleNamespace(Batch=stub)
    torch = types.SimpleNamespace(cuda=types.SimpleNamespace(synchronize=lambda: None))
    args = types.SimpleNamespace(batch_instances=40)
    res = bench.run_batch_sharded(args, torch, q, rep)
    out.put((rank, res))
    rep.close()


def _two_bench_ranks(stub):
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_bench_rank_main, args=(r, 2, port, out, stub)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return res


def test_bench_batch_section_on_two_ranks():
    """bench.py's batch section with two ranks: both report the same job
    (all instances' gates over the slowest rank) and a balanced split, and
    rank 0 finds the reassembled results equal to a single-rank run."""
    pytest.importorskip("torch.distributed")
    (_, a), (_, b) = _two_bench_ranks(_StubBatch)
    assert a["ranks"] == b["ranks"] == 2 and a["instances"] == 40
    for k in ("c64", "c128"):
        assert a[k]["s"] == b[k]["s"] and a[k]["gates_per_s"] == a["total_gates"] / a[k]["s"]
        assert a[k]["matches_single_rank_run"] is True
        assert "matches_single_rank_run" not in b[k]
    assert a["max_over_mean_load"] < 1.5


def test_bench_batch_section_reports_a_mismatch():
    """A batch whose results depend on the batch around an instance gives
    different bits when split: rank 0's check reports it."""
    pytest.importorskip("torch.distributed")
    (_, a), _ = _two_bench_ranks(_PositionalStubBatch)
    for k in ("c64", "c128"):
        assert a[k]["matches_single_rank_run"] is False
