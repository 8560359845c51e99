"""Number-preserving backend on the GPU against the oracle's NP
restatement (full 2^n vector walked through generateLookup tables, as
src/qubits/np/*.cpp does).  The GPU stores only the C(n, w) amplitudes of
weight w; getState expands them, and every index outside the sector must be
exactly zero."""
import itertools

import numpy as np
import pytest

from conftest import bits, random_np_state

pytestmark = pytest.mark.gpu

NP_GATES = ("pauliZ", "rotateZ", "phase", "controlZ", "controlRotateZ", "controlPhase",
            "swap", "fswap", "npRotateX", "npRotateY", "npHadamard")
ONE = {"pauliZ", "rotateZ", "phase"}


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
@pytest.mark.parametrize("n,w", [(2, 1), (4, 1), (6, 3), (8, 4), (9, 2), (10, 7)])
def test_np_gates_all_pairs(qsl, port, dtype, n, w):
    rng = np.random.default_rng(n * 31 + w)
    st = random_np_state(rng, n, w, dtype)
    gpu = qsl.QubitsNP(state=st, dtype=dtype)
    assert gpu.getNumOnes() == w
    cpu = port.PortNPQubits(n, w, fp32=dtype == np.complex64, state=st)
    for g in NP_GATES:
        if g in ONE:
            for t in range(n):
                a = rng.uniform(0, 2 * np.pi)
                gpu.gate(g, t, angle=a)
                cpu.gate(g, t, angle=a)
        else:
            for q1, q2 in itertools.permutations(range(n), 2):
                a = rng.uniform(0, 2 * np.pi)
                gpu.gate(g, q1, q2, a)
                cpu.gate(g, q1, q2, a)
    out = gpu.getState()
    assert np.array_equal(bits(out), bits(cpu.state))


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_np_measurement(qsl, port, dtype):
    rng = np.random.default_rng(3)
    n, w = 14, 6
    st = random_np_state(rng, n, w, dtype)
    gpu = qsl.QubitsNP(state=st, dtype=dtype)
    cpu = port.PortNPQubits(n, w, fp32=dtype == np.complex64, state=st)
    for t in range(n):
        for o in (0, 1):
            assert gpu.prob(t, o) == cpu.prob(t, o)
    u = rng.random(4000)
    if dtype == np.complex64:
        u = u.astype(np.float32).astype(np.float64)
    assert np.array_equal(gpu.sample_shots(u), cpu.sample_all(u))
    for t in (0, 7, 13):
        uu = float(np.float32(rng.random())) if dtype == np.complex64 else rng.random()
        assert gpu.measure(t, uu) == cpu.measure(t, uu)
    assert np.array_equal(bits(gpu.getState()), bits(cpu.state))


def test_np_construction_semantics(qsl):
    q = qsl.QubitsNP(6, 2)
    st = q.getState()
    assert st[0b11] == 1 and np.count_nonzero(st) == 1          # np.cpp:69-79
    assert q.num_stored() == 15
    q.setNumOnes(3)
    assert q.getNumOnes() == 3 and q.getState()[0b111] == 1
    with pytest.raises(qsl.LogicError):
        qsl.QubitsNP(5, 0)
    with pytest.raises(qsl.LogicError):
        qsl.QubitsNP(5, 5)
    bad = np.zeros(64, dtype=np.complex128)
    bad[0b11] = bad[0b111] = 1 / np.sqrt(2)
    with pytest.raises(qsl.LogicError):
        q.setState(bad)
    q.setBasisState(0b101010)
    assert q.getNumOnes() == 3 and q.getState()[0b101010] == 1
    with pytest.raises(qsl.LogicError):
        q.pauliX(0)


def test_np_edge_angles_match_oracle(qsl, port):
    """Number-preserving gates at angles whose coefficients leave the
    integer products' range (exact zero or tiny sines) and near pi."""
    rng = np.random.default_rng(7)
    n, w = 10, 4
    st = random_np_state(rng, n, w)
    gpu = qsl.QubitsNP(state=st)
    cpu = port.PortNPQubits(n, w, state=st)
    for a in (0.0, 2 * np.pi, 1e-30, np.pi, -np.pi, 2.0**-70):
        for g in ("phase", "rotateZ"):
            gpu.gate(g, 3, None, a)
            cpu.gate(g, 3, None, a)
        for g in ("controlPhase", "controlRotateZ", "npRotateX", "npRotateY"):
            gpu.gate(g, 0, n - 1, a)
            cpu.gate(g, 0, n - 1, a)
    assert np.array_equal(bits(gpu.getState()), bits(cpu.state))
