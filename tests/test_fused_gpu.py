"""The precision form: gates queued on a complex64 state, fused into dense
blocks of up to k qubits and applied in FP32; norms, probabilities and the
sampling CDF in FP64.  Checked against the FP64 oracle: infidelity
1 - |<psi_64|psi_fused>|^2 <= 1e-6 (the target of the precision form) and the
largest amplitude error; sampling on the fused state matches the oracle's
double-accumulated CDF (the reference's Dist for float states) shot for shot."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ALL1 = ("pauliX", "pauliY", "pauliZ", "hadamard", "phase", "rotateX", "rotateY", "rotateZ")
ALL2 = ("controlNot", "controlY", "controlZ", "controlRotateX", "controlRotateY",
        "controlRotateZ", "controlPhase", "controlHadamard", "swap", "fswap", "npRotateX",
        "npRotateY", "npHadamard")


def random_circuit(rng, n, length):
    circ = []
    for _ in range(length):
        if rng.random() < 0.6:
            circ.append((str(rng.choice(ALL1)), int(rng.integers(n)), None,
                         float(rng.uniform(0, 2 * np.pi))))
        else:
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            circ.append((str(rng.choice(ALL2)), a, b, float(rng.uniform(0, 2 * np.pi))))
    return circ


@pytest.mark.parametrize("k,tc", [(2, False), (3, False), (4, False), (5, False), (5, True)])
def test_fused_matches_fp64(qsl, port, k, tc):
    from qsl_gb300 import workloads
    rng = np.random.default_rng(40 + k)
    n = 14
    circ = random_circuit(rng, n, 400) + workloads.layered_mixed(n, 6, 5 + k)
    gpu = qsl.Qubits(n, dtype=np.complex64)
    gpu.set_fusion(k)
    gpu.set_fusion_tc(tc)
    workloads.apply(gpu, circ)
    ref = port.PortQubits(n)
    workloads.apply(ref, circ)
    st = gpu.getState().astype(np.complex128)
    blocks = gpu.fused_blocks()
    assert 0 < blocks < len(circ)
    fid = abs(np.vdot(ref.state, st)) ** 2 / (np.vdot(st, st).real * np.vdot(ref.state, ref.state).real)
    assert 1 - fid <= 1e-6, 1 - fid
    assert np.abs(st - ref.state).max() <= 2e-5
    for t in range(n):
        assert abs(gpu.prob(t, 0) - ref.prob(t, 0)) <= 1e-5


def test_fused_sampling_uses_fp64_cdf(qsl, port):
    from qsl_gb300 import workloads
    n = 13
    gpu = qsl.Qubits(n, dtype=np.complex64)
    gpu.set_fusion(5)
    workloads.apply(gpu, workloads.layered_mixed(n, 10, 77))
    st = gpu.getState()
    cpu = port.PortQubits(n, fp32=True, state=st)
    u = np.random.default_rng(3).random(5000).astype(np.float32).astype(np.float64)
    assert np.array_equal(gpu.sample_shots(u), cpu.sample_all(u))
    # probabilities summed in FP64: the exact sequential double sum of the
    # float |a|^2 terms
    for t in (0, 6, 12):
        s = 0.0
        idx = np.arange(1 << n)
        sel = st[(idx >> t) & 1 == 1]
        for p in (sel.real.astype(np.float32) ** 2 + sel.imag.astype(np.float32) ** 2):
            s += float(p)
        assert gpu.prob(t, 1) == s


def test_fusion_flushes_before_reads_and_rejects_c128(qsl):
    q = qsl.Qubits(8, dtype=np.complex64)
    q.set_fusion(4)
    q.hadamard(0)
    q.controlNot(0, 5)
    st = q.getState()
    assert abs(st[0] - 2 ** -0.5) < 1e-7 and abs(st[0b100001] - 2 ** -0.5) < 1e-7
    with pytest.raises(qsl.LogicError):
        qsl.Qubits(4).set_fusion(3)
    with pytest.raises(qsl.LogicError):
        q.set_fusion(6)
