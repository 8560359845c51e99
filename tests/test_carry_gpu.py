"""Gate outputs whose two rounded products both round up to a power of two.

A rotation or phase output is RN(RN(a*c) +- RN(b*s)).  When a's significand
times c's lies just below a power of two, RN(a*c) carries out to that power,
and when both products of one output do so with the same exponent and the
same effective sign, the integer-pipe sum meets its largest operands.  On
random states this happens about once in 2^100 outputs, so these tests build
states from such operands: every real and imaginary part is +-ma * 2^k with
ma * m(c) just below a power of two, for one of the gate's constants c, and
scaled so that every such product rounds to +-2^-8.  Each gate runs on a
fresh copy of the state with every output on the integer pipes (mask 15),
with the default split and with the FP64 pipe alone, and must give the
oracle's bits."""
import math
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import bits

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
E_TARGET = -8
ANGLE = None      # set by the first call of angle()

GATES1 = ("rotateX", "rotateY", "rotateZ", "phase")
GATES2 = ("controlRotateX", "controlRotateY", "controlRotateZ", "controlPhase", "npRotateX",
          "npRotateY")
NP_GATES = ("rotateZ", "phase", "controlPhase", "controlRotateZ", "npRotateX", "npRotateY")

SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, {root!r})
import qsl_gb300 as q
d = np.load({inp!r})
cls = q.QubitsNP if {np_sim!r} else q.Qubits
out = []
for g, a, b in zip(d["names"], d["q1"], d["q2"]):
    sim = cls(state=d["state"])
    sim.gate(str(g), int(a), None if int(b) < 0 else int(b), float(d["angle"]))
    out.append(sim.getState())
np.save({out!r}, np.stack(out))
"""


def significand(c: float):
    """(m, e) with |c| = m * 2^(e - 52), m a 53-bit integer."""
    f, e = math.frexp(abs(c))
    return int(f * (1 << 53)), e - 1


def carry_operand(c: float, top: int):
    """The positive double a whose product with c rounds up to 2^E_TARGET
    from just below it, or None: a's significand ma has ma * m(c) in
    [2^(105+top) - 2^(51+top), 2^(105+top))."""
    mc, ec = significand(c)
    hi = 1 << (105 + top)
    lo = hi - (1 << (51 + top))
    ma = -(-lo // mc)
    if not ((1 << 52) <= ma < (1 << 53)) or ma * mc >= hi:
        return None
    ea = E_TARGET - ec - 1 - top
    a = math.ldexp(ma, ea - 52)
    assert a * abs(c) == 2.0 ** E_TARGET and ma * mc != hi
    return a


def constants(theta: float):
    return (math.cos(theta / 2), math.sin(theta / 2), math.cos(theta), math.sin(theta))


def angle():
    """The first angle on a fixed grid whose four constants all have carry
    operands."""
    global ANGLE
    if ANGLE is None:
        for k in range(1, 100000):
            th = 0.3 + k * 1e-4
            if all(carry_operand(c, 0) or carry_operand(c, 1) for c in constants(th)):
                ANGLE = th
                break
    assert ANGLE is not None
    return ANGLE


def operands(theta: float):
    ops = [a for c in constants(theta) for top in (0, 1) if (a := carry_operand(c, top)) is not None]
    assert len(ops) >= 4
    return np.array(ops)


def crafted_state(rng, n: int, theta: float, support=None) -> np.ndarray:
    ops = operands(theta)
    size = 1 << n if support is None else support.size
    re = rng.choice(ops, size) * rng.choice([-1.0, 1.0], size)
    im = rng.choice(ops, size) * rng.choice([-1.0, 1.0], size)
    if support is None:
        return re + 1j * im
    v = np.zeros(1 << n, dtype=np.complex128)
    v[support] = re + 1j * im
    return v


def run_gpu(tmp_path, state, names, q1, q2, theta, mask_env, np_sim=False):
    inp, out = str(tmp_path / "in.npz"), str(tmp_path / "out.npy")
    np.savez(inp, state=state, names=np.array(names), q1=np.array(q1), q2=np.array(q2),
             angle=np.array(theta))
    env = dict(os.environ, **mask_env)
    r = subprocess.run([sys.executable, "-c", SCRIPT.format(root=ROOT, inp=inp, out=out, np_sim=np_sim)],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return np.load(out)


def test_crafted_state_hits_the_carry_case():
    """Sanity of the construction (CPU only): in rotateX's output
    a0.re * cos + a1.im * sin, many pairs have both products equal to
    +2^-8 or both to -2^-8."""
    th = angle()
    st = crafted_state(np.random.default_rng(1), 10, th)
    c, s = math.cos(th / 2), math.sin(th / 2)
    a0, a1 = st[0::2], st[1::2]
    p, q = a0.real * c, a1.imag * s
    hits = (np.abs(p) == 2.0 ** E_TARGET) & (p == q)
    assert hits.sum() >= 8


MASKS = [dict(QSLC_EMU_MASK="15", QSLC_EMU_MASK_DIAG="3", QSLC_EMU_MASK_NP="15",
              QSLC_EMU_MASK_NP_DIAG="3"),
         dict(),
         dict(QSLC_EMU_MASK="0", QSLC_EMU_MASK_DIAG="0", QSLC_EMU_MASK_NP="0",
              QSLC_EMU_MASK_NP_DIAG="0")]


@pytest.mark.gpu
@pytest.mark.parametrize("mask", range(len(MASKS)))
def test_carry_products_full_simulator(qsl, port, tmp_path, mask):
    rng = np.random.default_rng(20 + mask)
    n = 11
    th = angle()
    st = crafted_state(rng, n, th)
    names, q1, q2 = [], [], []
    for g in GATES1 + GATES2:
        for _ in range(3):
            a, b = (int(v) for v in rng.choice(n, 2, replace=False))
            names.append(g)
            q1.append(a)
            q2.append(b if g in GATES2 else -1)
    got = run_gpu(tmp_path, st, names, q1, q2, th, MASKS[mask])
    for i, (g, a, b) in enumerate(zip(names, q1, q2)):
        cpu = port.PortQubits(n, state=st)
        cpu.gate(g, a, None if b < 0 else b, th)
        assert np.array_equal(bits(got[i]), bits(cpu.state)), (g, a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("mask", range(len(MASKS)))
def test_carry_products_np_simulator(qsl, port, tmp_path, mask):
    rng = np.random.default_rng(40 + mask)
    n, w = 11, 5
    th = angle()
    support = port.generate_lookup(n, w).astype(np.int64)
    st = crafted_state(rng, n, th, support)
    names, q1, q2 = [], [], []
    for g in NP_GATES:
        for _ in range(3):
            a, b = (int(v) for v in rng.choice(n, 2, replace=False))
            names.append(g)
            q1.append(a)
            q2.append(-1 if g in ("phase", "rotateZ") else b)
    got = run_gpu(tmp_path, st, names, q1, q2, th, MASKS[mask], np_sim=True)
    for i, (g, a, b) in enumerate(zip(names, q1, q2)):
        cpu = port.PortNPQubits(n, w, state=st)
        cpu.gate(g, a, None if b < 0 else b, th)
        assert np.array_equal(bits(got[i]), bits(cpu.state)), (g, a, b)
