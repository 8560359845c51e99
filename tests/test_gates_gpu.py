"""Gate parity on the GPU: every gate, every qubit (pair), both precisions,
compared bit for bit with the oracle (the reference's arithmetic, restated).

The reference's own gate tests apply each gate to a random 8-qubit state and
compare with a dense operator to 1e-6/1e-8 (src/gtest/gates.cpp:313-876);
here the bar is identical bits, with the 1e-12 bound of the FP64 path also
asserted on its own."""
import itertools

import numpy as np
import pytest

from conftest import bits, random_state

pytestmark = pytest.mark.gpu

GATES1 = ("pauliX", "pauliY", "pauliZ", "hadamard", "phase", "rotateX", "rotateY", "rotateZ")
GATES2 = ("controlNot", "controlY", "controlZ", "controlRotateX", "controlRotateY",
          "controlRotateZ", "controlPhase", "controlHadamard", "swap", "fswap", "npRotateX",
          "npRotateY", "npHadamard")
TOL = {np.complex128: 1e-12, np.complex64: 1e-5}


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
@pytest.mark.parametrize("n", [1, 2, 3, 5, 9])
def test_one_qubit_gates_all_targets(qsl, port, dtype, n):
    rng = np.random.default_rng(100 + n)
    st = random_state(rng, n, dtype)
    gpu = qsl.Qubits(state=st, dtype=dtype)
    cpu = port.PortQubits(n, fp32=dtype == np.complex64, state=st)
    for g in GATES1:
        for t in range(n):
            a = rng.uniform(0, 2 * np.pi)
            gpu.gate(g, t, angle=a)
            cpu.gate(g, t, angle=a)
    out = gpu.getState()
    assert np.abs(out - cpu.state).max() <= TOL[dtype]
    assert np.array_equal(bits(out), bits(cpu.state))


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
@pytest.mark.parametrize("n", [2, 3, 6, 8])
def test_two_qubit_gates_all_pairs(qsl, port, dtype, n):
    rng = np.random.default_rng(200 + n)
    st = random_state(rng, n, dtype)
    gpu = qsl.Qubits(state=st, dtype=dtype)
    cpu = port.PortQubits(n, fp32=dtype == np.complex64, state=st)
    for g in GATES2:
        for q1, q2 in itertools.permutations(range(n), 2):
            a = rng.uniform(0, 2 * np.pi)
            gpu.gate(g, q1, q2, a)
            cpu.gate(g, q1, q2, a)
    out = gpu.getState()
    assert np.abs(out - cpu.state).max() <= TOL[dtype]
    assert np.array_equal(bits(out), bits(cpu.state))


def test_random_circuit_16q(qsl, port):
    rng = np.random.default_rng(7)
    n = 16
    gpu = qsl.Qubits(n)
    cpu = port.PortQubits(n)
    for _ in range(300):
        if rng.random() < 0.5:
            g = str(rng.choice(GATES1))
            t = int(rng.integers(n))
            a = rng.uniform(0, 2 * np.pi)
            gpu.gate(g, t, angle=a)
            cpu.gate(g, t, angle=a)
        else:
            g = str(rng.choice(GATES2))
            q1, q2 = (int(x) for x in rng.choice(n, 2, replace=False))
            a = rng.uniform(0, 2 * np.pi)
            gpu.gate(g, q1, q2, a)
            cpu.gate(g, q1, q2, a)
    out = gpu.getState()
    assert np.array_equal(bits(out), bits(cpu.state))


def test_invalid_arguments_raise(qsl):
    q = qsl.Qubits(4)
    with pytest.raises(qsl.LogicError):
        q.pauliX(4)
    with pytest.raises(qsl.LogicError):
        q.controlNot(1, 1)
    with pytest.raises(qsl.LogicError):
        q.setState(np.zeros(8, dtype=np.complex128))
    q2 = qsl.Qubits(5)
    with pytest.raises(qsl.LogicError):
        q.assign(q2)


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_edge_angles_match_oracle(qsl, port, dtype):
    """Angles whose coefficients leave the integer products' range -- an
    exact zero sine (angle 0, 2 pi), a sine below 2^-64 (1e-30) -- run
    every output on the FP64 pipe; angles near pi give a cosine near
    2^-54, inside the range.  All must give the oracle's bits."""
    rng = np.random.default_rng(99)
    n = 11
    st = random_state(rng, n, dtype)
    gpu = qsl.Qubits(state=st, dtype=dtype)
    cpu = port.PortQubits(n, fp32=dtype == np.complex64, state=st)
    angles = (0.0, 2 * np.pi, 1e-30, -1e-30, np.pi, -np.pi, 3 * np.pi, 1e-10, 2.0**-70)
    for a in angles:
        for g in ("rotateX", "rotateY", "rotateZ", "phase"):
            for t in (0, 5, n - 1):
                gpu.gate(g, t, None, a)
                cpu.gate(g, t, None, a)
        for g in ("controlRotateX", "controlRotateY", "controlRotateZ", "controlPhase",
                  "npRotateX", "npRotateY"):
            gpu.gate(g, 0, n - 1, a)
            cpu.gate(g, 0, n - 1, a)
    assert np.array_equal(bits(gpu.getState()), bits(cpu.state))
