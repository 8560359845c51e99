"""Grouped one-qubit gates: the library holds a one-qubit gate back until
the next call; a one-qubit gate on another qubit joins it in one sweep
(k_group2), anything else releases it alone.  Every sequence must give the
oracle's bits, whatever call follows a held gate: another one-qubit gate
on the same or another qubit, a two-qubit gate, a probability, a copy, an
assignment, a state read, or a call that replaces the state."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import bits, random_state

pytestmark = pytest.mark.gpu

ONE = ("pauliX", "pauliY", "pauliZ", "hadamard", "phase", "rotateX", "rotateY", "rotateZ")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_both(qsl, port, st, ops, dtype):
    gpu = qsl.Qubits(state=st, dtype=dtype)
    cpu = port.PortQubits(int(st.size).bit_length() - 1, fp32=dtype == np.complex64, state=st)
    for op in ops:
        if op[0] == "prob":
            assert gpu.prob(op[1], 1) == cpu.prob(op[1], 1)
        else:
            gpu.gate(*op)
            cpu.gate(*op)
    return gpu, cpu


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
@pytest.mark.parametrize("n", [2, 5, 12])
def test_grouped_sequences_match_oracle(qsl, port, dtype, n):
    rng = np.random.default_rng(70 + n)
    st = random_state(rng, n, dtype)
    ops = []
    for _ in range(60):
        r = rng.random()
        q = int(rng.integers(n))
        if r < 0.6:                                   # another one-qubit gate
            ops.append((str(rng.choice(ONE)), q, None, float(rng.uniform(0, 2 * np.pi))))
        elif r < 0.7 and ops and ops[-1][0] != "prob":  # the same qubit again
            ops.append((str(rng.choice(ONE)), ops[-1][1], None, float(rng.uniform(0, 2 * np.pi))))
        elif r < 0.85:
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            ops.append((str(rng.choice(["controlNot", "controlPhase", "swap", "controlRotateY"])), a, b,
                        float(rng.uniform(0, 2 * np.pi))))
        else:
            ops.append(("prob", q))
    gpu, cpu = run_both(qsl, port, st, ops, dtype)
    assert np.array_equal(bits(gpu.getState()), bits(cpu.state))


def test_held_gate_before_copy_assign_and_replace(qsl, port):
    """A gate held back when the state is copied, assigned from, or
    replaced: the copy and the assignment see it applied; set_state and
    reset discard it with the state it would have changed."""
    rng = np.random.default_rng(5)
    n = 9
    st = random_state(rng, n)
    gpu, cpu = run_both(qsl, port, st, [("rotateY", 3, None, 0.7)], np.complex128)
    cp = gpu.copy()
    assert np.array_equal(bits(cp.getState()), bits(cpu.state))
    other = qsl.Qubits(n)
    gpu.gate("hadamard", 4)                           # held again
    cpu.gate("hadamard", 4)
    other.assign(gpu)
    assert np.array_equal(bits(other.getState()), bits(cpu.state))
    gpu.gate("rotateX", 2, None, 1.1)                 # held, then discarded
    fresh = random_state(rng, n)
    gpu.setState(fresh)
    cpu2 = port.PortQubits(n, state=fresh)
    gpu.gate("rotateZ", 6, None, 0.3)
    gpu.gate("rotateZ", 7, None, 0.4)                 # grouped with the previous one
    cpu2.gate("rotateZ", 6, None, 0.3)
    cpu2.gate("rotateZ", 7, None, 0.4)
    assert np.array_equal(bits(gpu.getState()), bits(cpu2.state))


SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, {root!r})
import qsl_gb300 as q
d = np.load({inp!r})
sim = q.Qubits(state=d["state"])
l0 = sim.launches()
for g, a, x in zip(d["names"], d["q1"], d["ang"]):
    sim.gate(str(g), int(a), None, float(x))
np.save({out!r}, sim.getState())
print(sim.launches() - l0)
"""


def test_grouping_off_gives_the_same_bits(tmp_path):
    """QSLC_GROUP=0 launches every gate alone; the bits are the same and
    grouping halves the launches of a run of one-qubit gates."""
    rng = np.random.default_rng(8)
    n = 14
    st = random_state(rng, n)
    names = np.array([str(rng.choice(ONE)) for _ in range(40)])
    q1 = np.array([k % n for k in range(40)])
    ang = rng.uniform(0, 2 * np.pi, 40)
    inp = str(tmp_path / "in.npz")
    np.savez(inp, state=st, names=names, q1=q1, ang=ang)
    outs, launches = [], []
    for grp in ("1", "0"):
        out = str(tmp_path / f"out{grp}.npy")
        r = subprocess.run([sys.executable, "-c", SCRIPT.format(root=ROOT, inp=inp, out=out)],
                           env=dict(os.environ, QSLC_GROUP=grp), capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        outs.append(np.load(out))
        launches.append(int(r.stdout.split()[-1]))
    assert np.array_equal(bits(outs[0]), bits(outs[1]))
    assert launches[1] == 40 and launches[0] == 20
