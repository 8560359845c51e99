"""Hadamard outputs whose quotient by RN(sqrt(2)) lies next to a rounding
decision.

The integer-pipe division estimates x / RN(sqrt 2) from a 96-bit
reciprocal and declines, to the FP64 pipe's division, the quotients whose
fraction it cannot place on one side of one half.  On random states that is
about one output in 2^39, so this test builds the dividends: with my the
odd significand of RN(sqrt 2), a significand mx with mx * 2^k = r (mod my)
(k = 52 when mx >= my, else 53) leaves the fraction r / my, which is
1 / (2 my) from one half for r = (my -+ 1) / 2.  It also builds exact
quotients (r = 0) and fractions just below the next integer (r = my - 1).

Every amplitude whose target bit is 0 gets such values (the partner is
zero, so each output divides one of them), and hadamard must give the
oracle's bits with the division on the integer pipes (mask 0) and with the
sums there too (mask 15)."""
import math
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import bits

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SQRT2 = math.sqrt(2)

SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, {root!r})
import qsl_gb300 as q
d = np.load({inp!r})
out = []
for t in d["targets"]:
    sim = q.Qubits(state=d["states"][len(out)])
    sim.hadamard(int(t))
    out.append(sim.getState())
np.save({out!r}, np.stack(out))
"""


def significands():
    """(mx, r) pairs for the residues (my - 1) / 2, (my + 1) / 2, 0, my - 1."""
    f, _ = math.frexp(SQRT2)
    my = int(f * (1 << 53))
    assert my & 1
    found = []
    for k in (52, 53):
        inv = pow(1 << k, -1, my)
        for r in ((my - 1) // 2, (my + 1) // 2, 0, my - 1):
            mx0 = r * inv % my
            for j in range(4):
                mx = mx0 + j * my
                if (1 << 52) <= mx < (1 << 53) and (mx < my) == (k == 53):
                    found.append((mx, r, my, k))
    return found


def values():
    return np.array([math.ldexp(mx, e - 52) for mx, _, _, _ in significands() for e in (-9, -8, -7)])


def test_dividends_sit_next_to_midpoints():
    """CPU only: the built significands give the fractions claimed, and at
    least one quotient on each side of a midpoint."""
    near = 0
    for mx, r, my, k in significands():
        assert (mx << k) % my == r
        frac = r / my
        if abs(frac - 0.5) < 1e-15:
            near += 1
    assert near >= 2


def crafted(rng, n, t):
    vals = values()
    st = np.zeros(1 << n, dtype=np.complex128)
    idx = np.array([i for i in range(1 << n) if not (i >> t) & 1])
    st[idx] = (rng.choice(vals, idx.size) * rng.choice([-1.0, 1.0], idx.size) +
               1j * rng.choice(vals, idx.size) * rng.choice([-1.0, 1.0], idx.size))
    return st


@pytest.mark.gpu
@pytest.mark.parametrize("mask", ["0", "15"])
def test_hadamard_near_midpoints(qsl, port, tmp_path, mask):
    rng = np.random.default_rng(int(mask) + 3)
    n = 9
    targets = [0, 3, 8]
    states = np.stack([crafted(rng, n, t) for t in targets])
    inp, out = str(tmp_path / "in.npz"), str(tmp_path / "out.npy")
    np.savez(inp, states=states, targets=np.array(targets))
    env = dict(os.environ, QSLC_EMU_MASK_H=mask)
    r = subprocess.run([sys.executable, "-c", SCRIPT.format(root=ROOT, inp=inp, out=out)],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got = np.load(out)
    for i, t in enumerate(targets):
        cpu = port.PortQubits(n, state=states[i])
        cpu.gate("hadamard", t, None, 0.0)
        assert np.array_equal(bits(got[i]), bits(cpu.state)), t
        # the quotients themselves, against the host's IEEE division
        keep = [j for j in range(1 << n) if not (j >> t) & 1]
        src, res = states[i][keep], got[i][keep]
        assert np.array_equal(res.real.view(np.uint64), (src.real / SQRT2).view(np.uint64))
        assert np.array_equal(res.imag.view(np.uint64), (src.imag / SQRT2).view(np.uint64))
