"""The phase-gate timing of qsl's examples/benchmark-np.cpp on the GPU.

For every number of ones 1 .. n-1: a random state of that weight, a random
phase per qubit, `reps` phase gates on every qubit, timed on the full
(Cuda) and the number-preserving (CudaNP) backends; the mean time per gate
in seconds goes into a Results table written in qsl's format, which qsl's
scripts/plot.py reads next to its own results/np_phase.csv.

    python -m qsl_gb300.benchmark_np [--nqubits 16] [--reps 1000] [--out np_phase_cuda.csv]

Like the reference, each timing is host wall time around the loop; the
device is synchronised at the end of the loop, so the figure is the time
per gate of a stream of gates, launch included.
"""
from __future__ import annotations

import argparse
import time

import numpy as np

from . import Qubits, QubitsNP
from .results import Results
from .workloads import weight_indices


def random_np_state(n: int, w: int, rng) -> np.ndarray:
    """A random normalised state supported on the basis indices of weight
    w, the role of makeRandomNPState (include/qsl/utils/random.hpp:117)."""
    v = np.zeros(1 << n, dtype=np.complex128)
    idx = weight_indices(n, w).astype(np.int64)
    v[idx] = rng.uniform(-1, 1, idx.size) + 1j * rng.uniform(-1, 1, idx.size)
    return v / np.linalg.norm(v)


def time_phase(sim, phases, reps: int) -> float:
    n = len(phases)
    sim.synchronize()
    t0 = time.perf_counter()
    for q in range(n):
        for _ in range(reps):
            sim.phase(q, phases[q])
    sim.synchronize()
    return (time.perf_counter() - t0) / (n * reps)


def run(nqubits: int = 16, reps: int = 1000, seed: int = 0) -> Results:
    rng = np.random.default_rng(seed)
    res = Results(["nones", "Cuda", "CudaNP"])
    res.addMeta("Testing the phase gate")
    full = Qubits(nqubits)
    for w in range(1, nqubits):
        state = random_np_state(nqubits, w, rng)
        phases = rng.uniform(0, 2 * np.pi, nqubits)
        full.setState(state)
        npsim = QubitsNP(state=state)
        res.addRow([w], [time_phase(full, phases, reps), time_phase(npsim, phases, reps)])
        del npsim
    return res


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--nqubits", type=int, default=16)
    ap.add_argument("--reps", type=int, default=1000)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default="np_phase_cuda.csv")
    a = ap.parse_args(argv)
    res = run(a.nqubits, a.reps, a.seed)
    res.writeToFile(a.out)
    res.print()


if __name__ == "__main__":
    main()
