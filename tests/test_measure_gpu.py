"""Measurement parity on the GPU: prob, measure, postselect, sample,
sampleAll and measureAll, bit for bit (probabilities) and shot for shot
(outcomes) against the oracle fed the same uniforms.

The reference tests these statistically (1000 samples, 0.1 tolerance,
src/gtest/measurements.cpp:20, :487-665); with the uniforms shared the
comparison can be exact."""
import numpy as np
import pytest

from conftest import bits, random_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
@pytest.mark.parametrize("n", [1, 4, 11, 14, 17])
def test_prob_bit_exact(qsl, port, dtype, n):
    rng = np.random.default_rng(n)
    st = random_state(rng, n, dtype)
    gpu = qsl.Qubits(state=st, dtype=dtype)
    cpu = port.PortQubits(n, fp32=dtype == np.complex64, state=st)
    for t in range(n):
        for o in (0, 1):
            assert gpu.prob(t, o) == cpu.prob(t, o), (t, o)


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
@pytest.mark.parametrize("n", [1, 3, 10, 15, 18])
def test_sample_all_shot_for_shot(qsl, port, dtype, n):
    rng = np.random.default_rng(30 + n)
    st = random_state(rng, n, dtype)
    gpu = qsl.Qubits(state=st, dtype=dtype)
    cpu = port.PortQubits(n, fp32=dtype == np.complex64, state=st)
    u = rng.random(5000)
    if dtype == np.complex64:
        u = u.astype(np.float32).astype(np.float64)
    a = gpu.sample_shots(u)
    b = cpu.sample_all(u)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_measure_postselect_sequence(qsl, port, dtype):
    rng = np.random.default_rng(5)
    n = 12
    st = random_state(rng, n, dtype)
    gpu = qsl.Qubits(state=st, dtype=dtype)
    cpu = port.PortQubits(n, fp32=dtype == np.complex64, state=st)
    for t in rng.permutation(n)[:8]:
        u = float(np.float32(rng.random())) if dtype == np.complex64 else rng.random()
        assert gpu.measure(int(t), u) == cpu.measure(int(t), u)
    assert np.array_equal(bits(gpu.getState()), bits(cpu.state))
    st = random_state(rng, n, dtype)
    gpu.setState(st)
    cpu.state[:] = st
    assert gpu.postselect(3, 1) == cpu.postselect(3, 1)
    assert np.array_equal(bits(gpu.getState()), bits(cpu.state))


def test_sample_counts_and_measure_all(qsl, port):
    rng = np.random.default_rng(9)
    n = 13
    st = random_state(rng, n)
    gpu = qsl.Qubits(state=st)
    cpu = port.PortQubits(n, state=st)
    u = rng.random(20000)
    assert gpu.sample(4, 20000, u) == [int(x) for x in cpu.sample(4, u)]
    uu = rng.random()
    assert gpu.measureAll(uu) == cpu.measure_all(uu)
    assert np.array_equal(gpu.getState(), cpu.state)


def test_adversarial_sums(qsl, port):
    """Equal magnitudes (every term an exact tie candidate), a sum that
    crosses several powers of two, zeros, and a tiny tail."""
    n = 16
    rng = np.random.default_rng(11)
    cases = []
    v = np.full(1 << n, 1.0 / np.sqrt(1 << n), dtype=np.complex128)       # uniform
    cases.append(v)
    v = np.zeros(1 << n, dtype=np.complex128)
    v[::3] = 1e-3 * (1 + rng.random(v[::3].size))                          # zeros between
    cases.append(v)
    v = (rng.random(1 << n) * 7.0).astype(np.complex128)                   # unnormalised, sum >> 1
    cases.append(v)
    v = np.geomspace(1, 1e-150, 1 << n).astype(np.complex128)               # wide range
    cases.append(v)
    v = np.zeros(1 << n, dtype=np.complex128)
    v[12345] = 1.0                                                          # basis state
    cases.append(v)
    for st in cases:
        gpu = qsl.Qubits(state=st)
        cpu = port.PortQubits(n, state=st)
        for t in (0, 5, n - 1):
            assert gpu.prob(t, 0) == cpu.prob(t, 0)
            assert gpu.prob(t, 1) == cpu.prob(t, 1)
        total = cpu.dist()[1][-1] if cpu.dist()[1].size else 0.0
        u = np.concatenate([rng.random(3000) * max(total, 1e-300), [total, np.nextafter(total, 0)]])
        assert np.array_equal(gpu.sample_shots(u), cpu.sample_all(u))


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
@pytest.mark.parametrize("n", [3, 12, 16])
def test_sample_all2_counts(qsl, port, dtype, n):
    """sampleAll2 (measure.cpp:237-267): sorted uniforms merged against an Fp
    running sum with a strict comparison; uniforms above the total counted
    nowhere."""
    rng = np.random.default_rng(60 + n)
    st = random_state(rng, n, dtype) * (0.9 if n == 12 else 1.0)    # total below 1: some uncounted
    gpu = qsl.Qubits(state=st, dtype=dtype)
    cpu = port.PortQubits(n, fp32=dtype == np.complex64, state=st)
    u = rng.random(6000)
    if dtype == np.complex64:
        u = u.astype(np.float32).astype(np.float64)
    counts = cpu.sample_all2(u)
    got = gpu.sampleAll2(6000, uniforms=u)
    assert len(got) == 1 << n
    assert np.array_equal(np.array([got[i] for i in range(1 << n)], dtype=np.uint64), counts)


def test_sample_all2_np(qsl, port):
    from conftest import random_np_state
    rng = np.random.default_rng(8)
    n, w = 12, 5
    st = random_np_state(rng, n, w)
    gpu = qsl.QubitsNP(state=st)
    cpu = port.PortNPQubits(n, w, state=st)
    u = rng.random(4000)
    counts = cpu.sample_all2(u)
    got = gpu.sampleAll2(4000, uniforms=u)
    keys = port.generate_lookup(n, w)
    assert sorted(got) == [int(k) for k in keys]
    assert np.array_equal(np.array([got[int(k)] for k in keys], dtype=np.uint64), counts)
