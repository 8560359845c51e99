"""The debug build: with -DQSLC_DEBUG_BOUNDS the plain sweeps check each
item's indices against the state, skip an item outside it and report the
first such index as QSLC_EINVAL at the next call that reads the state.
Through the ABI no index can leave the state (qubit indices are validated
before any launch), so a debug build must give the default build's bits
and report nothing, over every sweep form: grouped one-qubit gates, single
one-qubit and diagonal gates, controlled and number-preserving pairs,
fswap, controlZ and controlPhase."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import bits, random_state

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, {root!r})
import qsl_gb300 as q
if {lib!r}:
    q.lib({lib!r})
d = np.load({inp!r})
sim = q.Qubits(state=d["state"])
for g, a, b, x in zip(d["names"], d["q1"], d["q2"], d["ang"]):
    sim.gate(str(g), int(a), None if int(b) < 0 else int(b), float(x))
    if g == "fswap":
        sim.prob(int(a), 1)
np.save({out!r}, sim.getState())
"""


def debug_library(tmp_path) -> str:
    from qsl_gb300 import build as b
    b.build()
    obj = str(tmp_path / "gates_debug.o")
    lib = str(tmp_path / "libqslc_debug.so")
    src = os.path.join(b.CSRC, "gates.cu")
    r = subprocess.run([b.nvcc(), *b.ARCH, *b.NVCC_FLAGS, "-DQSLC_DEBUG_BOUNDS", "-c", src, "-o", obj],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    objs = [os.path.join(b.OBJ, f) for f in sorted(os.listdir(b.OBJ))
            if f.endswith(".o") and f != "gates.o"]
    cudalib = os.path.join(os.path.dirname(os.path.dirname(b.nvcc())), "lib64")
    r = subprocess.run([b.nvcc(), *b.ARCH, "-shared", "-o", lib, *objs, obj, "-lcudart", "-lpthread",
                        "-L", cudalib, "-Xlinker", "-rpath", "-Xlinker", cudalib],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return lib


def test_debug_bounds_build_gives_the_default_bits(tmp_path):
    rng = np.random.default_rng(61)
    n = 11
    st = random_state(rng, n)
    one = ("pauliX", "pauliY", "pauliZ", "hadamard", "phase", "rotateX", "rotateY", "rotateZ")
    two = ("controlNot", "controlZ", "controlPhase", "controlRotateY", "swap", "fswap", "npRotateX")
    names, q1, q2, ang = [], [], [], []
    for _ in range(80):
        if rng.random() < 0.6:
            names.append(str(rng.choice(one)))
            q1.append(int(rng.integers(n)))
            q2.append(-1)
        else:
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            names.append(str(rng.choice(two)))
            q1.append(a)
            q2.append(b)
        ang.append(float(rng.uniform(0, 2 * np.pi)))
    inp = str(tmp_path / "in.npz")
    np.savez(inp, state=st, names=np.array(names), q1=np.array(q1), q2=np.array(q2), ang=np.array(ang))
    outs = []
    for tag, lib in (("default", ""), ("debug", debug_library(tmp_path))):
        out = str(tmp_path / f"{tag}.npy")
        r = subprocess.run([sys.executable, "-c", SCRIPT.format(root=ROOT, lib=lib, inp=inp, out=out)],
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        outs.append(np.load(out))
    assert np.array_equal(bits(outs[0]), bits(outs[1]))
