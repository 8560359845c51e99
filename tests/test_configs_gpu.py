"""Parity at the benchmark configurations' own sizes.

The other GPU tests compare every kernel with the oracle on small states
(at most 18 qubits).  These run the workloads of the benchmark's five
configurations at their stated sizes, or at the largest size the oracle can
hold beside them, and compare with the oracle bit for bit:

* 20 qubits, 20 layers of one-qubit gates and controlNot pairings, every
  qubit's prob, measureAll on a copy and 10,000 shots (the whole of the
  plain Default-backend configuration);
* 30 qubits (16 GiB): the benchmark circuit's first layers, its 8 measured
  qubits and its 100,000-shot sampleAll;
* 31 qubits (32 GiB): one gate of every kernel family with the top qubit
  and qubit 0, prob and a measurement -- the top of the 32-bit index path;
* the number-preserving 28-qubit weight-14 state with its 2,000 gates;
* a sample of the batching form's own 4,096 instances, the 20-qubit ones
  included, out of the whole batch run;
* the precision form at 32 qubits against the plain FP64 path on the same
  GPU (the 64-bit index path of both; infidelity <= 1e-6).

Large states are compared in slices read through the state's device
address, so the host holds one copy (the oracle's) and not two.  The
the benchmark spec tolerance for the plain FP64 path is 1e-12 in amplitude; the
tests assert identical bits, which is stricter, and the 1e-12 bound
beside them."""
import os

import numpy as np
import pytest

from qsl_gb300 import workloads

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
SLICE = 1 << 26                                # amplitudes per device-to-host slice
BENCH_SEED = 20240601                          # bench.py's SEED


def assert_same_bits(sim, host: np.ndarray, tol=1e-12):
    """The GPU state equals `host` bit for bit (and so within `tol`),
    compared slice by slice through the device address."""
    sim.synchronize()
    dev = sim.device_view()
    uint = np.uint64 if host.dtype == np.complex128 else np.uint32
    assert dev.shape[0] == host.size
    worst = 0.0
    for at in range(0, host.size, SLICE):
        part = dev[at:at + SLICE].cpu().numpy().view(host.dtype).reshape(-1)
        ref = host[at:at + SLICE]
        if not np.array_equal(part.view(uint), ref.view(uint)):
            bad = np.nonzero(part.view(uint) != ref.view(uint))[0]
            raise AssertionError(f"{bad.size} words differ in slice at {at}, first at "
                                 f"amplitude {at + bad[0] // 2}")
        worst = max(worst, float(np.abs(part - ref).max()))
    assert worst <= tol


def apply_both(gpu, cpu, circ):
    for g in circ:
        gpu.gate(*g)
        cpu.gate(*g)


def test_config1_20_qubits_as_written(qsl, port):
    """20 qubits from |0..0>: 20 layers of per-qubit gates from {hadamard,
    rotateX, rotateY, rotateZ, phase} and controlNot on a random pairing;
    prob(q, 0/1) on every qubit, measureAll once on a copy, sampleAll(10000)
    from fixed uniforms."""
    n = 20
    circ = workloads.layered_cnot(n, 20, 2024)
    assert len(circ) == 20 * (n + n // 2)
    gpu = qsl.Qubits(n)
    cpu = port.PortQubits(n, nthreads=THREADS)
    apply_both(gpu, cpu, circ)
    assert_same_bits(gpu, cpu.state)
    for q in range(n):
        for o in (0, 1):
            assert gpu.prob(q, o) == cpu.prob(q, o), (q, o)
    u_all = float(workloads.uniforms(1, 2025)[0])
    g2 = gpu.copy()
    c2 = port.PortQubits(n, state=cpu.state)
    got = g2.measureAll(u_all)
    assert got == c2.measure_all(u_all)
    basis = np.zeros(1 << n, dtype=np.complex128)
    basis[got] = 1
    assert_same_bits(g2, basis)
    u = workloads.uniforms(10_000, 2026)
    assert np.array_equal(gpu.sample_shots(u), cpu.sample_all(u))
    assert_same_bits(gpu, cpu.state)        # sampling leaves the state alone


def test_config2_30_qubits_first_layers_measure_sample(qsl, port):
    """The benchmark's 30-qubit circuit (16 GiB state): its first two
    layers, then its 8 measured qubits with its uniforms, then its
    100,000-shot sampleAll -- the same seeds bench.py uses."""
    n = 30
    circ = workloads.layered_mixed(n, 40, BENCH_SEED)
    per = n + n // 2
    gpu = qsl.Qubits(n)
    cpu = port.PortQubits(n, nthreads=THREADS)
    apply_both(gpu, cpu, circ[:2 * per])
    assert_same_bits(gpu, cpu.state)
    rng = np.random.default_rng(BENCH_SEED)
    mq = [int(x) for x in rng.choice(n, 8, replace=False)]
    mu = workloads.uniforms(8, BENCH_SEED + 1)
    for q, u in zip(mq, mu):
        assert gpu.measure(q, float(u)) == cpu.measure(q, float(u)), q
    assert_same_bits(gpu, cpu.state)
    su = workloads.uniforms(100_000, BENCH_SEED + 2)
    assert np.array_equal(gpu.sample_shots(su), cpu.sample_all(su))


def test_31_qubits_every_kernel_family(qsl, port):
    """A 31-qubit state (32 GiB, the largest swept with 32-bit indices):
    dense after rotateY on every qubit, then each kernel family on the top
    qubit (30) and on qubit 0, prob on both, and one measurement."""
    n = 31
    rng = np.random.default_rng(31)
    prep = [("rotateY", q, None, float(rng.uniform(0.3, 2.8))) for q in range(n)]
    gates = [
        ("hadamard", 30, None, 0.0), ("rotateX", 0, None, 0.7), ("rotateZ", 30, None, 1.9),
        ("phase", 30, None, 2.3), ("pauliY", 0, None, 0.0), ("pauliZ", 30, None, 0.0),
        ("controlNot", 30, 0, 0.0), ("controlNot", 0, 30, 0.0),
        ("controlRotateY", 29, 30, 0.4), ("controlHadamard", 30, 1, 0.0),
        ("controlPhase", 30, 0, 1.1), ("controlZ", 0, 29, 0.0),
        ("swap", 30, 0, 0.0), ("npRotateX", 0, 30, 0.9), ("fswap", 30, 15, 0.0),
    ]
    gpu = qsl.Qubits(n)
    cpu = port.PortQubits(n, nthreads=THREADS)
    apply_both(gpu, cpu, prep + gates)
    assert_same_bits(gpu, cpu.state)
    for q in (0, 30):
        for o in (0, 1):
            assert gpu.prob(q, o) == cpu.prob(q, o), (q, o)
    assert gpu.measure(30, 0.37) == cpu.measure(30, 0.37)
    assert_same_bits(gpu, cpu.state)


def test_config3_np_28_qubits_weight_14_2000_gates(qsl, port):
    """The number-preserving configuration in full: 28 qubits of weight 14
    (C(28,14) = 40,116,600 stored amplitudes), a seeded complex Gaussian
    state on the sector, 2000 gates from {npRotateX, swap, phase,
    controlPhase} -- bench.py's seeds -- then prob on every qubit and
    10,000 shots."""
    n, w = 28, 14
    st = workloads.np_gaussian_state(n, w, BENCH_SEED + 6)
    circ = workloads.np_mix(n, 2000, BENCH_SEED + 7)
    gpu = qsl.QubitsNP(state=st)
    assert gpu.num_stored() == 40_116_600
    cpu = port.PortNPQubits(n, w, nthreads=THREADS, state=st)
    del st
    apply_both(gpu, cpu, circ)
    # the compressed layout holds the sector's amplitudes in ascending basis
    # order; the oracle's full vector must equal it there and be zero elsewhere
    idx = workloads.weight_indices(n, w)
    assert_same_bits(gpu, np.ascontiguousarray(cpu.state[idx]))
    outside = np.ones(1 << n, dtype=bool)
    outside[idx] = False
    assert not np.any(cpu.state[outside])
    del outside
    for q in range(n):
        for o in (0, 1):
            assert gpu.prob(q, o) == cpu.prob(q, o), (q, o)
    u = workloads.uniforms(10_000, BENCH_SEED + 10)
    assert np.array_equal(gpu.sample_shots(u), cpu.sample_all(u))


def _batch_reference(port, n, layers, angles, u, fp32):
    sim = port.PortQubits(n, fp32=fp32, nthreads=THREADS if n >= 16 else 1)
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
def test_config5_batch_sample_of_the_4096(qsl, port, dtype):
    """The batching form's own workload (bench.py's 4,096 instances, n in
    [10, 20], L in [4, 16], 1,024 shots each) run as one batch; 48 of its
    instances, the largest ones among them, against the oracle."""
    import types

    import bench
    _, ns, ls, _, angles, u = bench.batch_workload(types.SimpleNamespace(batch_instances=4096))
    nshots = bench.BATCH_SHOTS
    fp32 = dtype == np.complex64
    if fp32:       # the reference draws Fp angles and uniforms
        angles = angles.astype(np.float32).astype(np.float64)
        u = u.astype(np.float32).astype(np.float64)
    b = qsl.Batch(ns, ls, nshots, dtype=dtype)
    probs, shots = b.run(angles, u)
    at = np.concatenate([[0], np.cumsum(2 * ns.astype(np.int64) * ls)])
    rng = np.random.default_rng(4096)
    big = np.nonzero(ns == ns.max())[0][:4]
    pick = np.unique(np.concatenate([big, rng.choice(ns.size, 44, replace=False)]))
    assert ns[pick].max() == 20
    for i in pick:
        n, L = int(ns[i]), int(ls[i])
        p, sh = _batch_reference(port, n, L, angles[at[i]:at[i + 1]],
                                 u[i * nshots:(i + 1) * nshots], fp32)
        assert np.array_equal(probs[i], p), (i, n, L)
        assert np.array_equal(shots[i], sh), (i, n, L)


def test_config4_fused_32_qubits_against_fp64(qsl):
    """The precision form at its own size: 32 qubits, complex64 (32 GiB),
    five-qubit blocks on the tensor cores, against the plain FP64 path
    (64 GiB, bit for bit the reference by the tests above) over the first
    three layers of the 32-qubit circuit; infidelity <= 1e-6, computed on
    the GPU in slices."""
    torch = pytest.importorskip("torch")
    n = 32
    circ = workloads.layered_mixed(n, 60, BENCH_SEED + 4)[:3 * (n + n // 2)]
    ref = qsl.Qubits(n)
    workloads.apply(ref, circ)
    f = qsl.Qubits(n, dtype=np.complex64)
    f.set_fusion(5)
    f.set_fusion_tc(True)
    workloads.apply(f, circ)
    f.flush()
    assert f.fused_blocks() > 0
    ref.synchronize()
    f.synchronize()
    a, b = ref.device_view(), f.device_view()
    dot = torch.zeros(2, dtype=torch.float64, device="cuda")
    na = torch.zeros((), dtype=torch.float64, device="cuda")
    nb = torch.zeros((), dtype=torch.float64, device="cuda")
    worst = torch.zeros((), dtype=torch.float64, device="cuda")
    for at in range(0, 1 << n, SLICE):
        x = a[at:at + SLICE]
        y = b[at:at + SLICE].double()
        # <x|y> = sum (xr - i xi)(yr + i yi)
        dot[0] += (x[:, 0] * y[:, 0] + x[:, 1] * y[:, 1]).sum()
        dot[1] += (x[:, 0] * y[:, 1] - x[:, 1] * y[:, 0]).sum()
        na += (x * x).sum()
        nb += (y * y).sum()
        worst = torch.maximum(worst, (x - y).abs().max())
    fid = float((dot * dot).sum() / (na * nb))
    assert 1 - fid <= 1e-6, 1 - fid
    assert float(worst) <= 1e-5
    assert abs(float(na) - 1) <= 1e-9
