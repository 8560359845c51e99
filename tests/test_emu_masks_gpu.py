"""Every split of the dense gate arithmetic between the FP64 pipe and the
integer pipes gives the oracle's bits.

QSLC_EMU_MASK (rotations), QSLC_EMU_MASK_H (Hadamard) and
QSLC_EMU_MASK_DIAG (phase, controlPhase) choose, per output of an amplitude
pair or of a diagonal update and per item of a sweep iteration, how it is
computed: F (FP64 pipe), P (both products on the integer pipes, the sum on
the FP64 pipe), Q (one product on the integer pipes) or E (all of it on the
integer pipes), as letters ("PPPQ,PPPP,FFEE"), or in the older numeric form
(bit i set: output i in mode E).  The library reads them once per process,
so each setting runs in its own process.  The settings cover the compiled
patterns and ones that take the runtime-pattern kernels."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import bits, random_state

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DENSE = ("hadamard", "rotateX", "rotateY", "rotateZ", "phase", "controlRotateX",
         "controlRotateY", "controlRotateZ", "controlPhase", "controlHadamard", "npRotateX",
         "npRotateY", "npHadamard")

SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, {root!r})
import qsl_gb300 as q
d = np.load({inp!r})
sim = q.Qubits(state=d["state"])
for g, a, b, x in zip(d["names"], d["q1"], d["q2"], d["ang"]):
    sim.gate(str(g), int(a), None if int(b) < 0 else int(b), float(x))
np.save({out!r}, sim.getState())
"""


def circuit(rng, n, reps):
    names, q1, q2, ang = [], [], [], []
    for _ in range(reps):
        for g in DENSE:
            a, b = (int(v) for v in rng.choice(n, 2, replace=False))
            two = g.startswith(("control", "np"))
            names.append(g)
            q1.append(a)
            q2.append(b if two else -1)
            ang.append(float(rng.uniform(0, 2 * np.pi)))
    return np.array(names), np.array(q1), np.array(q2), np.array(ang)


@pytest.mark.parametrize("rot,had,diag", [("0", "0", "0"), ("1", "5", "2"), ("3,5,1", "15", "1,0,3"),
                                          ("5,5,1", "0", "1,1,0"), ("7", "3,1,0", "3"),
                                          ("15", "15", "3"), ("10,12,6", "9", "2,1"),
                                          ("PPPP", "FFFF", "PP"), ("PPPP,PPPP,PPPQ", "EFFF", "PQ"),
                                          ("PPPQ", "FFFF", "PQ,PP,PP"), ("PPQQ", "EEFF", "QQ"),
                                          ("QQQQ,PQEF,FEQP", "FEFE", "QP,EF,FQ"),
                                          ("EPQF", "EEEE", "EP,QE")])
def test_every_emulation_split_is_exact(qsl, port, tmp_path, rot, had, diag):
    rng = np.random.default_rng(len(rot) * 7 + len(diag) + 3 * len(had))
    n = 12
    st = random_state(rng, n)
    names, q1, q2, ang = circuit(rng, n, 6)
    inp, out = str(tmp_path / "in.npz"), str(tmp_path / "out.npy")
    np.savez(inp, state=st, names=names, q1=q1, q2=q2, ang=ang)
    env = dict(os.environ, QSLC_EMU_MASK=rot, QSLC_EMU_MASK_H=had, QSLC_EMU_MASK_DIAG=diag)
    r = subprocess.run([sys.executable, "-c", SCRIPT.format(root=ROOT, inp=inp, out=out)],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    cpu = port.PortQubits(n, state=st)
    for g, a, b, x in zip(names, q1, q2, ang):
        cpu.gate(str(g), int(a), None if int(b) < 0 else int(b), float(x))
    assert np.array_equal(bits(np.load(out)), bits(cpu.state))


NP_SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, {root!r})
import qsl_gb300 as q
d = np.load({inp!r})
sim = q.QubitsNP(state=d["state"])
for g, a, b, x in zip(d["names"], d["q1"], d["q2"], d["ang"]):
    sim.gate(str(g), int(a), None if int(b) < 0 else int(b), float(x))
np.save({out!r}, sim.getState())
"""
NP_GATES = ("phase", "rotateZ", "controlPhase", "controlRotateZ", "npRotateX", "npRotateY",
            "npHadamard")


@pytest.mark.parametrize("pair,diag,had", [("0", "0", "0"), ("15", "3", "15"), ("5,1,1", "1,0,0", "0"),
                                           ("6,9,3", "2,3,1", "5"), ("PPPQ", "PQ", "FFFF"),
                                           ("PPPP", "PP", "EEFF"), ("QQQQ,PQEF,FFPP", "QQ,EP,FF", "FFFF")])
def test_np_emulation_splits_are_exact(qsl, port, tmp_path, pair, diag, had):
    from conftest import random_np_state
    rng = np.random.default_rng(len(pair) + 3 * len(diag))
    n, w = 12, 5
    st = random_np_state(rng, n, w)
    names, q1, q2, ang = [], [], [], []
    for _ in range(8):
        for g in NP_GATES:
            a, b = (int(v) for v in rng.choice(n, 2, replace=False))
            names.append(g)
            q1.append(a)
            q2.append(-1 if g in ("phase", "rotateZ") else b)
            ang.append(float(rng.uniform(0, 2 * np.pi)))
    inp, out = str(tmp_path / "in.npz"), str(tmp_path / "out.npy")
    np.savez(inp, state=st, names=np.array(names), q1=np.array(q1), q2=np.array(q2), ang=np.array(ang))
    env = dict(os.environ, QSLC_EMU_MASK_NP=pair, QSLC_EMU_MASK_NP_DIAG=diag, QSLC_EMU_MASK_H=had)
    r = subprocess.run([sys.executable, "-c", NP_SCRIPT.format(root=ROOT, inp=inp, out=out)],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    cpu = port.PortNPQubits(n, w, state=st)
    for g, a, b, x in zip(names, q1, q2, ang):
        cpu.gate(g, a, None if b < 0 else b, x)
    assert np.array_equal(bits(np.load(out)), bits(cpu.state))


@pytest.mark.parametrize("rot,diag", [("PPPQ,PPPQ,PPPF", "PQ,PQ,PP"), ("QQQQ,PQEF,FEQP", "QP,EF,FQ")])
def test_staged_sweeps_are_exact(qsl, port, tmp_path, rot, diag):
    """With QSLC_BULK=1 the one-qubit sweeps of 8 to 31 qubits stage their
    amplitudes through shared memory (bulk copies, mbarriers) instead of
    the register kernels; they must give the same bits, for low targets
    (one copied run per tile) and high ones (two runs)."""
    rng = np.random.default_rng(len(rot) + 5 * len(diag))
    n = 12
    st = random_state(rng, n)
    names, q1, q2, ang = circuit(rng, n, 4)
    inp, out = str(tmp_path / "in.npz"), str(tmp_path / "out.npy")
    np.savez(inp, state=st, names=names, q1=q1, q2=q2, ang=ang)
    env = dict(os.environ, QSLC_BULK="1", QSLC_EMU_MASK=rot, QSLC_EMU_MASK_DIAG=diag)
    r = subprocess.run([sys.executable, "-c", SCRIPT.format(root=ROOT, inp=inp, out=out)],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    cpu = port.PortQubits(n, state=st)
    for g, a, b, x in zip(names, q1, q2, ang):
        cpu.gate(str(g), int(a), None if int(b) < 0 else int(b), float(x))
    assert np.array_equal(bits(np.load(out)), bits(cpu.state))


SCRIPT_DTYPE = r"""
import sys, numpy as np
sys.path.insert(0, {root!r})
import qsl_gb300 as q
d = np.load({inp!r})
sim = q.Qubits(state=d["state"], dtype=d["state"].dtype)
for g, a, x in zip(d["names"], d["q1"], d["ang"]):
    sim.gate(str(g), int(a), None, float(x))
np.save({out!r}, sim.getState())
"""

PAIR1 = ("pauliX", "pauliY", "hadamard", "rotateX", "rotateY", "rotateZ")


def _run_pair1(tmp_path, tag, st, names, q1, ang, env):
    inp, out = str(tmp_path / f"in_{tag}.npz"), str(tmp_path / f"out_{tag}.npy")
    np.savez(inp, state=st, names=names, q1=q1, ang=ang)
    r = subprocess.run([sys.executable, "-c", SCRIPT_DTYPE.format(root=ROOT, inp=inp, out=out)],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return np.load(out)


@pytest.mark.parametrize("n", [5, 6, 11])
@pytest.mark.parametrize("rot,had", [("PPPQ,PPPQ,PPPF", "FFFF"), ("QQQQ,PQEF,FEQP", "FEFE"), ("0", "0")])
def test_warp_exchange_sweeps_are_exact(qsl, port, tmp_path, n, rot, had):
    """With QSLC_SHFL=1 the one-qubit pair gates on targets 0-4 take each
    pair's partner amplitude from another lane of the warp (k_pair1_shfl)
    instead of loading both members in one thread.  Every target 0-4 and
    every pair gate, with several splits between the pipes: complex128
    gives the oracle's bits, complex64 the register sweeps' bits.  A
    uniform state gives pairs of equal amplitudes, whose Hadamard
    difference is an exact zero (+0 in the reference)."""
    rng = np.random.default_rng(100 * n + len(rot) + len(had))
    names, q1, ang = [], [], []
    for _ in range(3):
        for g in PAIR1:
            for t in rng.permutation(min(n, 6)):
                names.append(g)
                q1.append(int(t))
                ang.append(float(rng.uniform(0, 2 * np.pi)))
    names, q1, ang = np.array(names), np.array(q1), np.array(ang)
    env = dict(os.environ, QSLC_EMU_MASK=rot, QSLC_EMU_MASK_H=had)
    st = random_state(rng, n)
    got = _run_pair1(tmp_path, "c128", st, names, q1, ang, dict(env, QSLC_SHFL="1"))
    cpu = port.PortQubits(n, state=st)
    for g, a, x in zip(names, q1, ang):
        cpu.gate(str(g), int(a), None, float(x))
    assert np.array_equal(bits(got), bits(cpu.state))
    st64 = random_state(rng, n, np.complex64)
    got64 = _run_pair1(tmp_path, "c64s", st64, names, q1, ang, dict(env, QSLC_SHFL="1"))
    reg64 = _run_pair1(tmp_path, "c64r", st64, names, q1, ang, dict(env, QSLC_SHFL="0"))
    assert np.array_equal(got64.view(np.uint32), reg64.view(np.uint32))
    flat = np.full(1 << n, (1 + 1j) / np.sqrt(2.0 ** (n + 1)), dtype=np.complex128)
    got = _run_pair1(tmp_path, "flat", flat, names, q1, ang, dict(env, QSLC_SHFL="1"))
    cpu = port.PortQubits(n, state=flat)
    for g, a, x in zip(names, q1, ang):
        cpu.gate(str(g), int(a), None, float(x))
    assert np.array_equal(bits(got), bits(cpu.state))
