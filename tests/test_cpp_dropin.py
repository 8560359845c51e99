"""The C++ drop-in, qsl::Qubits<qsl::cuda_type, Fp> (include/qsl/qubits/cuda.hpp).

CPU: it satisfies qsl's own concepts -- compiled against qsl's headers where
they are present, and against the standalone declarations everywhere.
GPU: a C++ program drives a circuit through the class exactly as a qsl user
would; its state, probabilities and sampleAll counts match the oracle."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from conftest import bits

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "tests", "cpp")
REF_INC = os.path.join(oracle.REF_SRC, "include") if oracle.REF_SRC else ""


def gxx(*args):
    r = subprocess.run(["g++", "-std=c++20", *args], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_concepts_standalone():
    gxx("-fsyntax-only", "-I", os.path.join(ROOT, "include"), os.path.join(CPP, "concepts_check.cpp"))


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_INC, "qsl")), reason="qsl headers absent")
def test_concepts_with_qsl_headers():
    gxx("-fsyntax-only", "-DWITH_QSL_HEADERS", "-I", os.path.join(ROOT, "include"), "-I", REF_INC,
        os.path.join(CPP, "concepts_check.cpp"))


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_INC, "qsl")), reason="qsl headers absent")
def test_verify_checkers_instantiate_and_link(qsl, tmp_path):
    """qsl::Verify with every checker of qsl's framework, CUDA backends as the
    second simulator, compiled against qsl's headers and linked against qsl's
    Default/NP implementation (oracle/_ref) and libqslc.  Running it needs
    those headers and a GPU on one machine."""
    import oracle
    oracle.build(reference=True)
    libdir = os.path.dirname(qsl.LIB_PATH)
    refdir = os.path.dirname(oracle.REF_SO)
    gxx("-O1", "-fopenmp", "-I", os.path.join(ROOT, "include"), "-I", REF_INC,
        os.path.join(CPP, "verify_check.cpp"), "-o", str(tmp_path / "verify_check"),
        "-L", libdir, "-lqslc", "-L", refdir, "-lqslref", f"-Wl,-rpath,{libdir}:{refdir}")


def build_drop_in(qsl, tmp):
    exe = os.path.join(tmp, "drop_in")
    libdir = os.path.dirname(qsl.LIB_PATH)
    gxx("-O2", "-I", os.path.join(ROOT, "include"), os.path.join(CPP, "drop_in.cpp"), "-o", exe,
        "-L", libdir, "-lqslc", f"-Wl,-rpath,{libdir}")
    return exe


def test_drop_in_links(qsl, tmp_path):
    assert os.path.exists(build_drop_in(qsl, str(tmp_path)))


@pytest.mark.gpu
@pytest.mark.parametrize("fp32", [False, True])
def test_drop_in_runs_like_the_oracle(qsl, port, tmp_path, fp32):
    from qsl_gb300 import workloads
    exe = build_drop_in(qsl, str(tmp_path))
    n, seed, shots = 11, 4242, 3000
    circ = workloads.layered_cnot(n, 6, 99)
    rng = np.random.default_rng(1)
    extra = [("controlRotateY", 3, 8, 0.7), ("fswap", 0, 10, 0.0), ("npHadamard", 9, 2, 0.0),
             ("controlHadamard", 5, 1, 0.0), ("pauliY", 7, None, 0.0)]
    circ = circ + extra
    if fp32:
        circ = [(g, a, b, float(np.float32(x))) for g, a, b, x in circ]
    path = os.path.join(str(tmp_path), "c.txt")
    with open(path, "w") as f:
        for g, a, b, x in circ:
            f.write(f"{g} {a} {-1 if b is None else b} {x!r}\n")
    out = os.path.join(str(tmp_path), "o.bin")
    args = [exe, path, out, str(n), str(seed), str(shots)] + (["f32"] if fp32 else [])
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = open(out, "rb").read()
    dt, rdt = (np.complex64, np.float32) if fp32 else (np.complex128, np.float64)
    off = 0
    st = np.frombuffer(raw, dtype=dt, count=1 << n, offset=off); off += st.nbytes
    probs = np.frombuffer(raw, dtype=rdt, count=2 * n, offset=off); off += probs.nbytes
    u = np.frombuffer(raw, dtype=rdt, count=shots, offset=off); off += u.nbytes
    pairs = np.frombuffer(raw, dtype=np.uint64, offset=off).reshape(-1, 2)
    sim = port.PortQubits(n, fp32=fp32)
    workloads.apply(sim, circ)
    assert np.array_equal(bits(st), bits(sim.state))
    assert np.array_equal(probs, np.array([sim.prob(t, o) for t in range(n) for o in (0, 1)], dtype=rdt))
    k, c = np.unique(sim.sample_all(u), return_counts=True)
    got = {int(a): int(b) for a, b in pairs if a != np.uint64(2**64 - 1)}
    assert got == {int(a): int(b) for a, b in zip(k, c)}
