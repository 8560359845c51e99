"""The batching form against the oracle, instance by instance: every
circuit's probabilities and shots are the bits the reference's Default
backend gives for the same gate calls and uniforms, in complex128 and in
complex64, for states in shared memory and states in the global arena."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def reference_instance(port, n, layers, angles, u, fp32):
    sim = port.PortQubits(n, fp32=fp32)
    a = angles.reshape(layers, n, 2)
    for l in range(layers):
        for q in range(n):
            sim.gate("rotateY", q, None, a[l, q, 0])
        for q in range(n):
            sim.gate("rotateZ", q, None, a[l, q, 1])
        for q in range(n - 1):
            sim.gate("controlNot", q, q + 1)
    probs = np.array([[sim.prob(q, 0), sim.prob(q, 1)] for q in range(n)])
    return probs, sim.sample_all(u)


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_batch_matches_oracle(qsl, port, dtype):
    rng = np.random.default_rng(11)
    ns = np.array([2, 5, 10, 13, 14, 15, 16, 12, 3, 11], dtype=np.uint32)
    ls = rng.integers(1, 6, ns.size).astype(np.uint32)
    nshots = 257
    b = qsl.Batch(ns, ls, nshots, dtype=dtype)
    angles = rng.uniform(0, 2 * np.pi, b.angle_count)
    fp32 = dtype == np.complex64
    if fp32:
        angles = angles.astype(np.float32).astype(np.float64)
    u = rng.random(ns.size * nshots)
    if fp32:
        u = u.astype(np.float32).astype(np.float64)
    for rep in range(2):                 # the graph replays
        probs, shots = b.run(angles, u)
        at = 0
        for i, (n, L) in enumerate(zip(ns, ls)):
            cnt = 2 * int(n) * int(L)
            p, sh = reference_instance(port, int(n), int(L), angles[at:at + cnt],
                                       u[i * nshots:(i + 1) * nshots], fp32)
            at += cnt
            assert np.array_equal(probs[i], p), (rep, i, n)
            assert np.array_equal(shots[i], sh), (rep, i, n)


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_every_launch_shape_matches_oracle(qsl, port, dtype):
    """Each launch shape the autotuner can choose -- shared-memory tiles of
    64 or 128 KB, 512 or 1024 threads, one or two CTAs per SM -- gives the
    oracle's bits, including instances of twice the tile's qubits (the
    two-pass path keeping no low qubits whole) and instances that fit a
    tile exactly."""
    import os
    rng = np.random.default_rng(21)
    fp32 = dtype == np.complex64
    k = 14 if fp32 else 13
    ns = np.array([2 * (k - 1), 18, k + 1, k, k - 1, 9, 2], dtype=np.uint32)
    ls = np.array([1, 2, 2, 2, 1, 3, 2], dtype=np.uint32)
    nshots = 300
    b = qsl.Batch(ns, ls, nshots, dtype=dtype)
    angles = rng.uniform(0, 2 * np.pi, b.angle_count)
    u = rng.random(ns.size * nshots)
    if fp32:
        angles = angles.astype(np.float32).astype(np.float64)
        u = u.astype(np.float32).astype(np.float64)
    want, at = [], 0
    for i, (n, L) in enumerate(zip(ns, ls)):
        cnt = 2 * int(n) * int(L)
        sim = port.PortQubits(int(n), fp32=fp32, nthreads=os.cpu_count() or 1)
        a = angles[at:at + cnt].reshape(int(L), int(n), 2)
        for l in range(int(L)):
            for q in range(int(n)):
                sim.gate("rotateY", q, None, a[l, q, 0])
            for q in range(int(n)):
                sim.gate("rotateZ", q, None, a[l, q, 1])
            for q in range(int(n) - 1):
                sim.gate("controlNot", q, q + 1)
        want.append((np.array([[sim.prob(q, 0), sim.prob(q, 1)] for q in range(int(n))]),
                     sim.sample_all(u[i * nshots:(i + 1) * nshots])))
        at += cnt
    shapes = b.shapes()
    assert len(shapes) >= 3
    for th, tl, c in shapes:
        b.set_shape(th, tl, c)
        assert b.shape()["tile_log2"] == tl
        probs, shots = b.run(angles, u)
        for i in range(ns.size):
            assert np.array_equal(probs[i], want[i][0]), (th, tl, c, i)
            assert np.array_equal(shots[i], want[i][1]), (th, tl, c, i)
    ms = b.autotune(angles, u)
    assert ms > 0 and tuple(b.shape()[x] for x in ("threads", "tile_log2", "ctas_per_sm")) in shapes
    probs, shots = b.run(angles, u)
    assert all(np.array_equal(probs[i], want[i][0]) for i in range(ns.size))


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_batch_sampling_on_exact_and_tied_sums(qsl, port, dtype):
    """The sampling CDFs walk in rounds within one binade, adding the term
    that leaves it on its own (k_batch_cdf).  Angles drawn from multiples of
    pi/4 make states with many equal and exactly zero |a|^2 terms -- exact
    partial sums, ties, leading zeros -- and uniforms sit on the
    reference's own partial sums and just above them; every shot must be
    the oracle's."""
    rng = np.random.default_rng(31)
    fp32 = dtype == np.complex64
    ns = np.array([3, 6, 9, 12, 14, 15], dtype=np.uint32)
    ls = np.array([1, 2, 1, 2, 1, 2], dtype=np.uint32)
    nshots = 200
    b = qsl.Batch(ns, ls, nshots, dtype=dtype)
    angles = rng.choice(np.array([0.0, 0.5, 1.0, 1.5, 0.25]) * np.pi, b.angle_count)
    if fp32:
        angles = angles.astype(np.float32).astype(np.float64)
    us, at = [], 0
    want = []
    for i, (n, L) in enumerate(zip(ns, ls)):
        n, L = int(n), int(L)
        cnt = 2 * n * L
        sim = port.PortQubits(n, fp32=fp32)
        a = angles[at:at + cnt].reshape(L, n, 2)
        at += cnt
        for l in range(L):
            for q in range(n):
                sim.gate("rotateY", q, None, a[l, q, 0])
            for q in range(n):
                sim.gate("rotateZ", q, None, a[l, q, 1])
            for q in range(n - 1):
                sim.gate("controlNot", q, q + 1)
        st = sim.state
        re, im = st.real, st.imag
        p = (re * re + im * im).astype(np.float64)       # RN(RN(re^2) + RN(im^2)) in the state's type
        cdf = np.cumsum(p)                                # sequential, in index order
        pick = cdf[rng.integers(0, cdf.size, nshots // 2)]
        u = np.concatenate([pick, np.nextafter(pick, 1.0)[: nshots // 4],
                            rng.random(nshots - nshots // 2 - nshots // 4)])
        u = np.clip(u, 0.0, np.nextafter(1.0, 0.0))
        if fp32:
            u = u.astype(np.float32).astype(np.float64)
        us.append(u)
        want.append(sim.sample_all(u))
    probs, shots = b.run(angles, np.concatenate(us))
    for i in range(ns.size):
        assert np.array_equal(shots[i], want[i]), (i, int(ns[i]))
