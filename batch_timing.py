#!/usr/bin/env python3
"""Device time of the batching kernel on a sub-batch of the benchmark's
batching workload (a bench tool beside bench.py).

The benchmark's batch is 4,096 ansatz instances (n uniform in [10, 20], L
in [4, 16]); this tool runs the instances `--first` of it plus the first
`--largest` 20-qubit ones, as one batch, `--repeat` times, and prints the
CUDA-event time of each run.  The first run is the ncu capture target of
one k_batch launch after a warm-up run (`-s 1 -c 1`):

    python batch_timing.py [--first 12] [--largest 4] [--dtype c128] [--repeat 3]
                           [--shape THREADS,TILE_LOG2,CTAS_PER_SM] [--max-qubits N]

Without `--shape` the batch keeps its default launch shape (1024 threads,
one CTA per SM, the larger tile); the benchmark's autotuner picks among
the shapes `Batch.shapes()` lists.
"""
from __future__ import annotations

import argparse
import os
import sys
import types

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def sub_batch(first: int, largest: int, max_qubits: int | None = None):
    """Indices of the chosen instances (ascending) and the sub-batch's
    qubit counts, layer counts, angles and uniforms.  With `max_qubits`,
    the instances of more qubits among the first ones are left out (the
    batch's arena, two buffers of the largest state per CTA, shrinks with
    it)."""
    import bench
    from qsl_gb300 import batch_shards as bs
    _, ns, ls, _, angles, u = bench.batch_workload(types.SimpleNamespace(batch_instances=4096))
    head = np.arange(first)
    if max_qubits is not None:
        head = head[ns[head] <= max_qubits]
    idx = np.unique(np.concatenate([head, np.nonzero(ns == ns.max())[0][:largest]]))
    return idx, bs.select(ns, ls, angles, u, bench.BATCH_SHOTS, idx)


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--first", type=int, default=12)
    ap.add_argument("--largest", type=int, default=4)
    ap.add_argument("--dtype", choices=["c128", "c64"], default="c128")
    ap.add_argument("--repeat", type=int, default=3)
    ap.add_argument("--shape", default=None, help="threads,tile_log2,ctas_per_sm")
    ap.add_argument("--max-qubits", type=int, default=None,
                    help="leave out the instances of more qubits among the first ones")
    a = ap.parse_args(argv)
    if a.first < 0 or a.largest < 0 or a.first + a.largest == 0 or a.first > 4096:
        ap.error("choose at least one instance, at most 4096 of the first ones")
    shape = None
    if a.shape is not None:
        try:
            shape = tuple(int(v) for v in a.shape.split(","))
        except ValueError:
            shape = ()
        if len(shape) != 3:
            ap.error("--shape takes three integers: threads,tile_log2,ctas_per_sm")
    import torch

    import bench
    import qsl_gb300 as q
    idx, (sn, sl, sa, su) = sub_batch(a.first, a.largest, a.max_qubits)
    if idx.size == 0:
        ap.error("no instance is left")
    b = q.Batch(sn, sl, bench.BATCH_SHOTS, dtype=np.complex128 if a.dtype == "c128" else np.complex64)
    if shape is not None:
        b.set_shape(*shape)
    for _ in range(a.repeat):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        b.run(sa, su)
        e1.record()
        torch.cuda.synchronize()
        print(f"{a.dtype} instances {idx.size} (n = {[int(x) for x in sn]}) shape {b.shape()}: "
              f"{e0.elapsed_time(e1):.1f} ms", flush=True)


if __name__ == "__main__":
    main()
