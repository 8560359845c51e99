"""The batching form split across ranks: one share of the instances per GPU.

Batch instances are independent circuits, so a batch shards with no data
exchange. Each rank runs its share as one batch on its own GPU. Rank 0 then
gathers the probabilities and shots and puts them back in instance order.

The cost of an instance is L * 2^n, its layers times its amplitudes. The
shares are assigned longest-first: each instance, in decreasing cost, goes
to the rank with the least cost so far. The ranks' totals then differ by at
most one instance's cost. The slowest rank is within 4/3 of the best
possible split (Graham's bound for this greedy).

    parts = partition_by_cost(instance_costs(ns, ls), world)
    mine = select(ns, ls, angles, uniforms, nshots, parts[rank])
    ... run `mine` as a Batch ...
    probs, shots = assemble(ns, nshots, parts, rep.gather((probs_r, shots_r)))
"""
from __future__ import annotations

import heapq

import numpy as np


def instance_costs(ns, ls) -> np.ndarray:
    """L * 2^n per instance, as int64."""
    n = np.asarray(ns, dtype=np.int64)
    L = np.asarray(ls, dtype=np.int64)
    return L << n


def partition_by_cost(costs, world: int) -> list:
    """Instance indices per rank (each ascending), longest first to the
    least-loaded rank; ties go to the lower rank, so every rank computes the
    same split."""
    if world < 1:
        raise ValueError("world must be at least 1")
    c = np.asarray(costs, dtype=np.int64)
    order = np.argsort(-c, kind="stable")
    heap = [(0, r) for r in range(world)]
    parts = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(int(i))
        heapq.heappush(heap, (load + int(c[i]), r))
    return [np.array(sorted(p), dtype=np.int64) for p in parts]


def _angle_offsets(ns, ls) -> np.ndarray:
    n = np.asarray(ns, dtype=np.int64)
    L = np.asarray(ls, dtype=np.int64)
    return np.concatenate([[0], np.cumsum(2 * n * L)])


def select(ns, ls, angles, uniforms, nshots: int, idx):
    """The sub-batch of instances `idx` (ascending): their qubit counts,
    layer counts, angles and uniforms, laid out as a Batch takes them."""
    ns = np.asarray(ns, dtype=np.uint32)
    ls = np.asarray(ls, dtype=np.uint32)
    idx = np.asarray(idx, dtype=np.int64)
    at = _angle_offsets(ns, ls)
    a = np.asarray(angles, dtype=np.float64)
    if a.size != at[-1]:
        raise ValueError(f"{a.size} angles for a batch that takes {at[-1]}")
    u = np.asarray(uniforms, dtype=np.float64).reshape(ns.size, nshots)
    sub_a = (np.concatenate([a[at[i]:at[i + 1]] for i in idx]) if idx.size
             else np.empty(0, dtype=np.float64))
    return ns[idx], ls[idx], sub_a, np.ascontiguousarray(u[idx]).reshape(-1)


def assemble(ns, nshots: int, parts, results):
    """Rank r's (probs, shots) for the instances parts[r], back in instance
    order: probs as a list of (n, 2) arrays, shots as (ninst, nshots)."""
    ninst = len(ns)
    probs = [None] * ninst
    shots = np.empty((ninst, nshots), dtype=np.uint64)
    seen = np.zeros(ninst, dtype=bool)
    for idx, (p, s) in zip(parts, results):
        s = np.asarray(s).reshape(len(idx), nshots)
        for k, i in enumerate(idx):
            if seen[i]:
                raise ValueError(f"instance {i} came back twice")
            seen[i] = True
            probs[i] = np.asarray(p[k])
            shots[i] = s[k]
    if not seen.all():
        raise ValueError(f"{int((~seen).sum())} instances did not come back")
    return probs, shots


def run_sharded(rep, ns, ls, nshots: int, angles, uniforms, runner):
    """Run this rank's share with `runner(ns, ls, angles, uniforms) ->
    (probs list, shots (k, nshots))` and gather every share.  Returns
    (probs, shots) in instance order on every rank, and this rank's part."""
    parts = partition_by_cost(instance_costs(ns, ls), rep.world)
    mine = parts[rep.rank]
    if mine.size:
        res = runner(*select(ns, ls, angles, uniforms, nshots, mine))
    else:
        res = ([], np.empty((0, nshots), dtype=np.uint64))
    gathered = rep.gather(([np.asarray(p) for p in res[0]], np.asarray(res[1])))
    probs, shots = assemble(ns, nshots, parts, gathered)
    return probs, shots, mine
