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


def test_prob_noalloc_rejects_oversized_states(qsl):
    L = qsl.lib()
    out = C.c_double()
    dummy = C.c_double(0.0)
    rc = L.qslc_prob_noalloc(C.addressof(dummy), 28, qsl.C128, 0, 0, None, C.byref(out))
    assert rc == qsl.EINVAL
    assert b"27" in L.qslc_last_error()
