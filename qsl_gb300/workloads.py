"""Seeded synthetic workloads (circuits and uniforms) of the benchmark
configurations.  The reference ships no benchmark circuits or datasets; these
generators produce the layered random circuits its hot path is measured on.

A circuit is a list of ``(gate, q1, q2, angle)`` tuples; ``q2`` is ``None``
for one-qubit gates and ``angle`` is 0.0 for gates without one.
"""
from __future__ import annotations

import numpy as np

ONE_QUBIT_MIX = ("hadamard", "rotateX", "rotateY", "rotateZ", "phase")


def layered_cnot(n: int, layers: int, seed: int):
    """Plain Default-backend circuit: per layer, per qubit one gate drawn from
    {hadamard, rotateX, rotateY, rotateZ, phase} with angle U[0, 2pi), then
    controlNot on a random perfect pairing of the qubits (a shuffled list
    taken two at a time)."""
    rng = np.random.default_rng(seed)
    circ = []
    for _ in range(layers):
        for q in range(n):
            g = ONE_QUBIT_MIX[int(rng.integers(len(ONE_QUBIT_MIX)))]
            a = float(rng.uniform(0, 2 * np.pi)) if g != "hadamard" else 0.0
            circ.append((g, q, None, a))
        perm = rng.permutation(n)
        for i in range(0, n - 1, 2):
            circ.append(("controlNot", int(perm[i]), int(perm[i + 1]), 0.0))
    return circ


def layered_mixed(n: int, layers: int, seed: int):
    """Layered circuit with mixed two-qubit gates: per layer one gate per
    qubit as in :func:`layered_cnot`, then n//2 two-qubit gates on a random
    perfect pairing, each controlNot or controlPhase (angle U[0, 2pi)) with a
    random orientation, so control and target range over high and low
    qubits alike."""
    rng = np.random.default_rng(seed)
    circ = []
    for _ in range(layers):
        for q in range(n):
            g = ONE_QUBIT_MIX[int(rng.integers(len(ONE_QUBIT_MIX)))]
            a = float(rng.uniform(0, 2 * np.pi)) if g != "hadamard" else 0.0
            circ.append((g, q, None, a))
        perm = rng.permutation(n)
        for i in range(0, n - 1, 2):
            c, t = int(perm[i]), int(perm[i + 1])
            if rng.random() < 0.5:
                circ.append(("controlNot", c, t, 0.0))
            else:
                circ.append(("controlPhase", c, t, float(rng.uniform(0, 2 * np.pi))))
    return circ


def np_mix(n: int, ngates: int, seed: int):
    """Number-preserving circuit: gates drawn from {npRotateX on a random
    pair, swap, phase, controlPhase} with angles U[0, 2pi)."""
    rng = np.random.default_rng(seed)
    circ = []
    for _ in range(ngates):
        k = int(rng.integers(4))
        if k == 0:
            q1, q2 = (int(x) for x in rng.choice(n, 2, replace=False))
            circ.append(("npRotateX", q1, q2, float(rng.uniform(0, 2 * np.pi))))
        elif k == 1:
            q1, q2 = (int(x) for x in rng.choice(n, 2, replace=False))
            circ.append(("swap", q1, q2, 0.0))
        elif k == 2:
            circ.append(("phase", int(rng.integers(n)), None, float(rng.uniform(0, 2 * np.pi))))
        else:
            q1, q2 = (int(x) for x in rng.choice(n, 2, replace=False))
            circ.append(("controlPhase", q1, q2, float(rng.uniform(0, 2 * np.pi))))
    return circ


def np_gaussian_state(n: int, w: int, seed: int, dtype=np.complex128) -> np.ndarray:
    """Complex Gaussian amplitudes on the weight-w sector, normalised; the
    full 2^n vector (zeros outside the sector)."""
    rng = np.random.default_rng(seed)
    idx = weight_indices(n, w)
    v = np.zeros(1 << n, dtype=np.complex128)
    v[idx] = rng.normal(size=idx.size) + 1j * rng.normal(size=idx.size)
    v /= np.linalg.norm(v)
    return v.astype(dtype)


def weight_indices(n: int, w: int) -> np.ndarray:
    """All n-bit integers with w set bits, ascending.  Built bit by bit: the
    k-bit integers of weight j are those of k-1 bits and weight j, then those
    of weight j-1 with bit k-1 set, so every list stays sorted; only weights
    that can still reach w are kept."""
    if w < 0 or w > n:
        return np.empty(0, dtype=np.int64)
    layer = {0: np.zeros(1, dtype=np.int64)}
    for k in range(1, n + 1):
        new = {}
        for j in range(max(0, w - (n - k)), min(k, w) + 1):
            parts = []
            if j in layer:
                parts.append(layer[j])
            if j - 1 in layer:
                parts.append(layer[j - 1] + (1 << (k - 1)))
            new[j] = np.concatenate(parts)
        layer = new
    return layer[w]


def uniforms(count: int, seed: int) -> np.ndarray:
    """Uniforms in (0, 1) standing in for the reference's random.getNum()."""
    u = np.random.default_rng(seed).random(count)
    u[u == 0.0] = np.nextafter(0.0, 1.0)
    return u


def apply(sim, circ) -> None:
    """Run a circuit on anything with ``gate(name, q1, q2, angle)``."""
    for g, q1, q2, a in circ:
        sim.gate(g, q1, q2, a)
