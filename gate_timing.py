#!/usr/bin/env python3
"""Device time of single gates on a dense state (a bench tool beside bench.py).

Prepares a state with no zero amplitudes (rotateY then rotateZ by a
random angle on every qubit, 2n sweeps), then applies each named gate to
each target qubit (one-qubit gates) or each control:target pair (two-qubit
gates) and prints its CUDA-event time on the simulator's stream, in
microseconds, with the algorithmic rate in GB/s (2 x 16 B x amplitudes the
reference's loop changes).  The preparation launches come first, so a
profiler that skips 2n launches of the one-qubit kernel captures the first
timed gate:

    python gate_timing.py [--qubits 26] [--gates hadamard,rotateX,hadamard,rotateX]
                          [--targets 3,9,15,21] [--pairs 0:5,5:0,20:21] [--angle 0.4]
                          [--repeat 1] [--grouped]

Each gate runs alone (the library's grouping of consecutive one-qubit
gates is switched off, QSLC_GROUP=0).  With --grouped, grouping stays on
and each timed window holds two one-qubit gates, on target t and on
target t + 1 (mod n), which run as one sweep; the rate is then the two
gates' algorithmic bytes over the window's time.

A gate on a state of zeros or of few nonzero amplitudes runs faster
than on a dense one (operands that are zero take a shorter path through
the exact arithmetic), so per-gate rates are measured here and not on
a freshly made |0...0>.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

TWO_QUBIT_AMPS = {"controlNot": 1, "controlY": 1, "controlRotateX": 1, "controlRotateY": 1,
                  "controlRotateZ": 1, "controlHadamard": 1, "swap": 1, "npRotateX": 1,
                  "npRotateY": 1, "npHadamard": 1, "controlZ": 2, "controlPhase": 2}
ONE_QUBIT_AMPS = {"hadamard": 0, "rotateX": 0, "rotateY": 0, "rotateZ": 0, "pauliX": 0,
                  "pauliY": 0, "phase": 1, "pauliZ": 1}


def alg_bytes(name: str, n: int) -> int:
    """2 x 16 B x the amplitudes the reference's loop changes (complex128)."""
    if name in ONE_QUBIT_AMPS:
        return 32 << (n - ONE_QUBIT_AMPS[name])
    return 32 << (n - TWO_QUBIT_AMPS[name])


def prepare_dense(sim, n: int, seed: int = 3) -> None:
    rng = np.random.default_rng(seed)
    for q in range(n):
        sim.rotateY(q, float(rng.uniform(0.3, 2.8)))
        sim.rotateZ(q, float(rng.uniform(0.3, 2.8)))


def parse_pairs(text: str, n: int):
    pairs = []
    for item in filter(None, text.split(",")):
        c, t = (int(x) for x in item.split(":"))
        if not (0 <= c < n and 0 <= t < n) or c == t:
            raise ValueError(f"pair {item} is not two distinct qubits of {n}")
        pairs.append((c, t))
    return pairs


def run(qubits: int, gates, targets, pairs, angle: float, repeat: int = 1, grouped: bool = False) -> dict:
    import torch

    from qsl_gb300 import Qubits

    stream = torch.cuda.Stream()
    sim = Qubits(qubits)
    sim.set_stream(stream.cuda_stream)
    prepare_dense(sim, qubits)
    sim.flush()
    torch.cuda.synchronize()
    out = {}
    for name in gates:
        one = name in ONE_QUBIT_AMPS
        where = [(t, None) for t in targets] if one else pairs
        pair = grouped and one
        times = []
        for q1, q2 in where:
            best = None
            for _ in range(repeat):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                sim.gate(name, q1, q2, angle)
                if pair:
                    sim.gate(name, (q1 + 1) % qubits, None, angle)
                sim.flush()
                e1.record(stream)
                torch.cuda.synchronize()
                us = e0.elapsed_time(e1) * 1e3
                best = us if best is None else min(best, us)
            times.append(round(best, 1))
        nb = alg_bytes(name, qubits) * (2 if pair else 1)
        gbs = [round(nb / (us * 1e-6) / 1e9) for us in times]
        out.setdefault(name, []).append({"us": times, "gbs": gbs, "where": where})
        print(name, where, times, "us", gbs, "GB/s", flush=True)
    return out


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--qubits", type=int, default=26)
    ap.add_argument("--gates", default="hadamard,rotateX,hadamard,rotateX")
    ap.add_argument("--targets", default="3,9,15,21")
    ap.add_argument("--pairs", default="0:5,5:0,1:9,20:21")
    ap.add_argument("--angle", type=float, default=0.4)
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--grouped", action="store_true",
                    help="time one-qubit gates two to a window, grouped into one sweep")
    a = ap.parse_args(argv)
    targets = [int(t) for t in a.targets.split(",")]
    if any(t < 0 or t >= a.qubits for t in targets):
        ap.error("every target must lie in [0, qubits)")
    try:
        pairs = parse_pairs(a.pairs, a.qubits)
    except ValueError as e:
        ap.error(str(e))
    gates = a.gates.split(",")
    for g in gates:
        if g not in ONE_QUBIT_AMPS and g not in TWO_QUBIT_AMPS:
            ap.error(f"unknown gate {g}")
    if not a.grouped:
        os.environ["QSLC_GROUP"] = "0"         # read once, at the library's first gate
    run(a.qubits, gates, targets, pairs, a.angle, max(1, a.repeat), a.grouped)


if __name__ == "__main__":
    main()
