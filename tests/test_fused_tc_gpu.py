"""Five-qubit fused blocks on the tensor cores (tcgen05.mma kind::tf32, 3xTF32
split, FP32 accumulation in tensor memory) against the same blocks on the CUDA
cores and against the FP64 oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(qsl, circ, n, tc):
    from qsl_gb300 import workloads
    q = qsl.Qubits(n, dtype=np.complex64)
    q.set_fusion(5)
    q.set_fusion_tc(tc)
    workloads.apply(q, circ)
    return q.getState().astype(np.complex128), q


def test_tensor_core_block_single(qsl):
    # one five-qubit block on a 12-qubit state: the smallest case the path takes
    circ = [("hadamard", q, None, 0.0) for q in range(5)] + [("rotateX", 2, None, 0.4),
                                                            ("controlNot", 0, 3, 0.0)]
    a, _ = run(qsl, circ, 12, False)
    b, q = run(qsl, circ, 12, True)
    assert q.fused_blocks() == 1
    assert np.abs(a - b).max() <= 1e-6


@pytest.mark.parametrize("n", [12, 15])
def test_tensor_core_blocks_match(qsl, port, n):
    from qsl_gb300 import workloads
    circ = workloads.layered_mixed(n, 12, 1234 + n)
    rng = np.random.default_rng(n)
    v = (rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n))
    v /= np.linalg.norm(v)
    outs = []
    for tc in (False, True):
        q = qsl.Qubits(state=v.astype(np.complex64), dtype=np.complex64)
        q.set_fusion(5)
        q.set_fusion_tc(tc)
        workloads.apply(q, circ)
        outs.append(q.getState().astype(np.complex128))
    assert np.abs(outs[0] - outs[1]).max() <= 2e-6
    ref = port.PortQubits(n, state=v)
    workloads.apply(ref, circ)
    fid = abs(np.vdot(ref.state, outs[1])) ** 2 / np.vdot(outs[1], outs[1]).real
    assert 1 - fid <= 1e-6
