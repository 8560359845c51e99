"""The resizeable backend (qsl's Type::Resize) on the GPU.

Fixtures: scripts of gates, addQubit, appendQubit, measureOut,
postselectOut, reallocateState and setState with a new size, run by the
reference itself (tests/golden/resize_*.npz); the GPU replays them and must
give the reference's state after every step, bit for bit in complex128.
The reference's own resize tests (src/gtest/resize-test.cpp:59-330) check
the same operations against dense projectors to 1e-6; here the bar is the
reference's bits, then size-independent properties at 24 qubits."""
import os

import numpy as np
import pytest

from conftest import bits, random_state

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def gpu_ops(sim):
    return dict(gate=sim.gate, add_qubit=sim.addQubit, append_qubit=sim.appendQubit,
                measure_out=lambda t, u: sim.measureOut(t, u), postselect_out=sim.postselectOut,
                reallocate=sim.reallocateState, set_state=sim.setState, get_state=sim.getState,
                prob=sim.prob, sample_all=sim.sample_shots)


@pytest.mark.parametrize("tag", ["c128", "c64"])
def test_resize_scripts_match_reference(qsl, tag):
    from golden.make_golden import load_cases
    from resize_replay import replay
    dtype = np.complex64 if tag == "c64" else np.complex128
    for name, c in load_cases(os.path.join(GOLD, f"resize_{tag}.npz")).items():
        sim = qsl.QubitsResize(state=c["init"], dtype=dtype)
        replay(c, gpu_ops(sim), dtype, exact=tag == "c128")


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_add_and_remove_every_position_against_oracle(qsl, port, dtype):
    rng = np.random.default_rng(5)
    n = 9
    st = random_state(rng, n, dtype)
    gpu = qsl.QubitsResize(state=st, dtype=dtype)
    cpu = port.PortResizeQubits(n, fp32=dtype == np.complex64, state=st)
    for t in range(n + 1):                 # addQubit at every position, then a gate on it
        gpu.addQubit(t)
        cpu.add_qubit(t)
        a = float(rng.uniform(0, 2 * np.pi))
        gpu.rotateY(t, a)
        cpu.gate("rotateY", t, None, a)
        assert np.array_equal(bits(gpu.getState()), bits(cpu.state)), t
    for t in range(2 * n, 1, -3):          # measureOut and postselectOut at spread positions
        t = min(t, gpu.nqubits - 1)
        u = float(rng.random())
        assert gpu.measureOut(t, u) == cpu.measure_out(t, u)
        assert np.array_equal(bits(gpu.getState()), bits(cpu.state))
        o = int(gpu.prob(0, 1) > 0.3)
        assert gpu.postselectOut(0, o) == cpu.postselect_out(0, o)
        assert np.array_equal(bits(gpu.getState()), bits(cpu.state))
    assert gpu.nqubits == cpu.n


def test_capacity_follows_the_reference(qsl):
    """dim_max doubles when a full state gains a qubit, stays when one is
    removed, and reallocateState trims it (resize.cpp:92-147)."""
    sim = qsl.QubitsResize(4)
    assert sim.capacity() == 16
    sim.appendQubit()
    assert sim.nqubits == 5 and sim.capacity() == 32
    sim.measureOut(2, 0.25)
    assert sim.nqubits == 4 and sim.capacity() == 32
    sim.addQubit(0)                        # fits: staged through scratch, no growth
    assert sim.nqubits == 5 and sim.capacity() == 32
    sim.measureOut(4, 0.5)
    sim.reallocateState()
    assert sim.capacity() == 16
    big = random_state(np.random.default_rng(1), 7)
    sim.setState(big)                      # any power-of-two size (resize.cpp:67-78)
    assert sim.nqubits == 7 and sim.capacity() >= 128
    assert np.array_equal(bits(sim.getState()), bits(big))
    with pytest.raises(qsl.LogicError):
        sim.setState(np.ones(12, dtype=np.complex128))
    other = qsl.QubitsResize(3)
    other.assign(sim)                      # assignment takes the other's size
    assert other.nqubits == 7 and np.array_equal(bits(other.getState()), bits(big))
    twin = sim.copy()
    twin.addQubit(3)
    assert sim.nqubits == 7 and twin.nqubits == 8


def test_resize_calls_rejected_elsewhere(qsl):
    plain = qsl.Qubits(4)
    with pytest.raises(qsl.LogicError):
        qsl.QubitsResize.addQubit(plain, 0)
    sim = qsl.QubitsResize(3)
    with pytest.raises(qsl.LogicError):
        sim.addQubit(5)                    # above the existing qubits
    one = qsl.QubitsResize(1)
    with pytest.raises(qsl.LogicError):
        one.measureOut(0, 0.5)             # the last qubit stays
    with pytest.raises(qsl.LogicError):
        plain.assign(sim)                  # different simulator kinds


@pytest.mark.parametrize("t", [0, 7, 23])
def test_add_then_collapse_out_is_identity_24q(qsl, t):
    """addQubit(t) then collapseOut(t, 0, 1) returns the same bits, and the
    added qubit reads prob 1 of |0> on the way, at 24 qubits (256 MiB)."""
    rng = np.random.default_rng(t)
    n = 24
    st = random_state(rng, n)
    sim = qsl.QubitsResize(state=st)
    sim.addQubit(t)
    assert sim.prob(t, 1) == 0.0 and sim.prob(t, 0) == pytest.approx(1.0, abs=1e-9)
    sim.collapseOut(t, 0, 1.0)
    assert sim.nqubits == n
    assert np.array_equal(bits(sim.getState()), bits(st))


def test_resize_after_fused_gates(qsl):
    """Queued fused gates are applied before the qubit count changes."""
    rng = np.random.default_rng(9)
    n = 14
    st = random_state(rng, n, np.complex64)
    a = qsl.QubitsResize(state=st, dtype=np.complex64)
    b = qsl.Qubits(state=st, dtype=np.complex64)
    a.set_fusion(4)
    b.set_fusion(4)
    for q in range(n):
        a.hadamard(q)
        b.hadamard(q)
    a.addQubit(5)
    ref = b.getState()
    got = a.getState()
    assert np.array_equal(bits(got[[i for i in range(1 << (n + 1)) if not i >> 5 & 1]]), bits(ref))
    assert not np.any(got[[i for i in range(1 << (n + 1)) if i >> 5 & 1]])
