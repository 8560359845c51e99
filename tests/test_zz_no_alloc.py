"""qslc_prob_noalloc: prob() for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc -- a framework whose memory pool owns
every device allocation, code that must not cause the device-wide
synchronisation an allocation can, a plugin in a process that has already
reserved the whole device.  This entry point takes the caller's device
amplitudes and works in a fixed, file-scope scratch array instead of
allocating.  Its answers must be the bits qslc_prob (the allocating entry
point) returns, on two calls in a row (the second call reuses the scratch
the first one left behind).

This file sorts last so a run that stops at the first failure has already
run every other test; it also passes on its own in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from conftest import random_state

pytestmark = pytest.mark.gpu


def test_prob_noalloc_matches_prob_twice(qsl):
    torch = pytest.importorskip("torch")
    L = qsl.lib()
    rng = np.random.default_rng(2718)
    for dtype, n in ((np.complex128, 13), (np.complex64, 9), (np.complex128, 20)):
        st = random_state(rng, n, dtype)
        ref = qsl.Qubits(state=st, dtype=dtype)
        code = qsl.C128 if dtype == np.complex128 else qsl.C64
        real = np.float64 if dtype == np.complex128 else np.float32
        dev = torch.from_numpy(st.view(real).copy()).cuda()     # caller-owned amplitudes
        stream = torch.cuda.current_stream().cuda_stream
        torch.cuda.synchronize()
        expect = {(t, o): ref.prob(t, o) for t in range(n) for o in (0, 1)}
        for call in range(2):
            for (t, o), want in expect.items():
                out = C.c_double(-1.0)
                rc = L.qslc_prob_noalloc(dev.data_ptr(), n, code, t, o, stream, C.byref(out))
                assert rc == 0, L.qslc_last_error()
                assert out.value == want, (dtype, n, call, t, o)


def test_prob_noalloc_at_its_largest_state(qsl):
    """27 qubits, the largest state the fixed scratch accepts (the carved
    scratch and the host arrays are at their fullest), in both dtypes."""
    torch = pytest.importorskip("torch")
    L = qsl.lib()
    rng = np.random.default_rng(27)
    n = 27
    for dtype, real, code in ((np.complex128, torch.float64, qsl.C128),
                              (np.complex64, torch.float32, qsl.C64)):
        gen = torch.Generator(device="cuda").manual_seed(int(rng.integers(1 << 30)))
        dev = torch.rand(2 << n, dtype=real, device="cuda", generator=gen) - 0.5
        dev /= torch.linalg.vector_norm(dev.double()).to(real)
        ref = qsl.Qubits(n, dtype=dtype)
        torch.cuda.synchronize()
        host = dev.cpu().numpy().view(dtype)
        ref.setState(host)
        stream = torch.cuda.current_stream().cuda_stream
        for call in range(2):
            for t, o in ((0, 0), (13, 1), (26, 0), (26, 1)):
                want = ref.prob(t, o)
                out = C.c_double(-1.0)
                rc = L.qslc_prob_noalloc(dev.data_ptr(), n, code, t, o, stream, C.byref(out))
                assert rc == 0, L.qslc_last_error()
                assert out.value == want, (dtype, call, t, o)
        del ref, dev, host
        torch.cuda.empty_cache()


def test_prob_noalloc_rejects_oversized_states(qsl):
    """Every qubit count outside [1, 27] is refused before any shift or CUDA
    call, including counts at and beyond the width of a 64-bit index."""
    L = qsl.lib()
    out = C.c_double()
    dummy = C.c_double(0.0)
    for n in (28, 40, 63, 64, 65, 70, 0):
        rc = L.qslc_prob_noalloc(C.addressof(dummy), n, qsl.C128, 0, 0, None, C.byref(out))
        assert rc == qsl.EINVAL, n
        assert b"27" in L.qslc_last_error(), n
