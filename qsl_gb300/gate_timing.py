"""Device time of single gates on a dense state.

Prepares a state with no zero amplitudes (rotateY then rotateZ by a
random angle on every qubit, 2n sweeps), then applies each named gate to
each target qubit and prints its CUDA-event time on the simulator's
stream, in microseconds. The preparation launches come first, so a
profiler that skips 2n launches of the one-qubit kernel captures the
first timed gate:

    python -m qsl_gb300.gate_timing [--qubits 26] [--gates hadamard,rotateX,hadamard,rotateX]
                                    [--targets 3,9,15,21] [--angle 0.4]

A gate on a state of zeros or of few nonzero amplitudes runs faster
than on a dense one (operands that are zero take a shorter path through
the exact arithmetic), so per-gate rates are measured here and not on
a freshly made |0...0>.
"""
from __future__ import annotations

import argparse

import numpy as np


def prepare_dense(sim, n: int, seed: int = 3) -> None:
    rng = np.random.default_rng(seed)
    for q in range(n):
        sim.rotateY(q, float(rng.uniform(0.3, 2.8)))
        sim.rotateZ(q, float(rng.uniform(0.3, 2.8)))


def run(qubits: int, gates, targets, angle: float) -> dict:
    import torch

    from . import Qubits

    stream = torch.cuda.Stream()
    sim = Qubits(qubits)
    sim.set_stream(stream.cuda_stream)
    prepare_dense(sim, qubits)
    torch.cuda.synchronize()
    out = {}
    for name in gates:
        times = []
        for t in targets:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sim.gate(name, t, None, angle)
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(round(e0.elapsed_time(e1) * 1e3, 1))
        out.setdefault(name, []).append(times)
        print(name, times, flush=True)
    return out


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--qubits", type=int, default=26)
    ap.add_argument("--gates", default="hadamard,rotateX,hadamard,rotateX")
    ap.add_argument("--targets", default="3,9,15,21")
    ap.add_argument("--angle", type=float, default=0.4)
    a = ap.parse_args(argv)
    targets = [int(t) for t in a.targets.split(",")]
    if any(t < 0 or t >= a.qubits for t in targets):
        ap.error("every target must lie in [0, qubits)")
    run(a.qubits, a.gates.split(","), targets, a.angle)


if __name__ == "__main__":
    main()
