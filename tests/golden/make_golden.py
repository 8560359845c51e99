"""Write the golden fixtures of tests/golden from the reference itself.

Runs qsl's own Default and NP backends (oracle/_ref/libqslref.so: the
reference sources compiled unmodified, random.cpp replaced by a seedable
stand-in that can be fed explicit uniforms) on seeded inputs and stores what
they return.  Needs the reference source tree (it builds oracle/_ref), so it
runs only where that tree exists; the fixtures it writes are committed and
travel to the GPU machine.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from qsl_gb300 import workloads  # noqa: E402

GATES1 = ("pauliX", "pauliY", "pauliZ", "hadamard", "phase", "rotateX", "rotateY", "rotateZ")
GATES2 = ("controlNot", "controlY", "controlZ", "controlRotateX", "controlRotateY",
          "controlRotateZ", "controlPhase", "controlHadamard", "swap", "fswap", "npRotateX",
          "npRotateY", "npHadamard")
NP_GATES1 = ("pauliZ", "rotateZ", "phase")
NP_GATES2 = ("controlZ", "controlRotateZ", "controlPhase", "swap", "fswap", "npRotateX",
             "npRotateY", "npHadamard")
ALL_NAMES = GATES1 + GATES2


def encode(circ):
    names = np.array([ALL_NAMES.index(g) for g, _, _, _ in circ], dtype=np.int32)
    q1 = np.array([a for _, a, _, _ in circ], dtype=np.int32)
    q2 = np.array([-1 if b is None else b for _, _, b, _ in circ], dtype=np.int32)
    ang = np.array([x for _, _, _, x in circ], dtype=np.float64)
    return names, q1, q2, ang


def decode(names, q1, q2, ang):
    return [(ALL_NAMES[int(k)], int(a), None if int(b) < 0 else int(b), float(x))
            for k, a, b, x in zip(names, q1, q2, ang)]


def random_circuit(rng, n, gates1, gates2, reps, fp32):
    circ = []
    for _ in range(reps):
        for g in gates1:
            a = float(rng.uniform(0, 2 * np.pi))
            if fp32:
                a = float(np.float32(a))
            circ.append((g, int(rng.integers(n)), None, a))
        for g in gates2:
            q1, q2 = (int(x) for x in rng.choice(n, 2, replace=False))
            a = float(rng.uniform(0, 2 * np.pi))
            if fp32:
                a = float(np.float32(a))
            circ.append((g, q1, q2, a))
    rng.shuffle(circ)
    return circ


def feed_map(ref, u):
    oracle.ref_feed_uniforms(u)
    m = ref.sample_all(len(u))
    assert oracle.ref_lib().qslref_uniforms_left() == 0
    keys = np.array(sorted(m), dtype=np.uint64)
    return keys, np.array([m[int(k)] for k in keys], dtype=np.uint64)


def uniforms(rng, count, fp32):
    u = rng.random(count)
    u[u == 0] = 0.5
    return u.astype(np.float32).astype(np.float64) if fp32 else u


def case_default(seed, n, fp32):
    rng = np.random.default_rng(seed)
    dt = np.complex64 if fp32 else np.complex128
    v = rng.uniform(-1, 1, 1 << n) + 1j * rng.uniform(-1, 1, 1 << n)
    init = (v / np.linalg.norm(v)).astype(dt)
    circ = random_circuit(rng, n, GATES1, GATES2, 3, fp32)
    ref = oracle.RefQubits("Default", fp32=fp32, state=init)
    workloads.apply(ref, circ)
    final = ref.get_state()
    probs = np.array([[ref.prob(t, o) for o in (0, 1)] for t in range(n)])
    u = uniforms(rng, 2000, fp32)
    keys, counts = feed_map(ref, u)
    u2 = uniforms(rng, 1500, fp32)
    oracle.ref_feed_uniforms(u2)
    m2 = ref.sample_all2(len(u2))
    counts2 = np.array([m2[i] for i in range(1 << n)], dtype=np.uint64)
    mu = uniforms(rng, 4, fp32)
    mq = rng.choice(n, 4, replace=False).astype(np.int32)
    outs = []
    for q, x in zip(mq, mu):
        oracle.ref_feed_uniforms([x])
        outs.append(ref.measure(int(q)))
    return dict(init=init, final=final, probs=probs, u=u, keys=keys, counts=counts,
                u2=u2, counts2=counts2,
                measure_qubits=mq, measure_u=mu, measure_out=np.array(outs, dtype=np.int32),
                after_measure=ref.get_state(), **dict(zip(("names", "q1", "q2", "ang"), encode(circ))))


def case_np(seed, n, w, fp32):
    rng = np.random.default_rng(seed)
    dt = np.complex64 if fp32 else np.complex128
    init = workloads.np_gaussian_state(n, w, seed, dt)
    circ = random_circuit(rng, n, NP_GATES1, NP_GATES2, 4, fp32)
    ref = oracle.RefQubits("NP", fp32=fp32, state=init)
    workloads.apply(ref, circ)
    final = ref.get_state()
    probs = np.array([[ref.prob(t, o) for o in (0, 1)] for t in range(n)])
    u = uniforms(rng, 2000, fp32)
    keys, counts = feed_map(ref, u)
    mu = uniforms(rng, 3, fp32)
    mq = rng.choice(n, 3, replace=False).astype(np.int32)
    outs = []
    for q, x in zip(mq, mu):
        oracle.ref_feed_uniforms([x])
        outs.append(ref.measure(int(q)))
    return dict(init=init, final=final, probs=probs, u=u, keys=keys, counts=counts,
                measure_qubits=mq, measure_u=mu, measure_out=np.array(outs, dtype=np.int32),
                after_measure=ref.get_state(), nones=np.int32(w),
                **dict(zip(("names", "q1", "q2", "ang"), encode(circ))))


def case_layered(seed, n, layers, nshots):
    """The 20-layer hadamard/rotation/phase + controlNot-pairing family,
    from |0...0>: state, every prob, measureAll on a copy, sampleAll."""
    rng = np.random.default_rng(seed + 1)
    circ = workloads.layered_cnot(n, layers, seed)
    ref = oracle.RefQubits("Default", nqubits=n)
    workloads.apply(ref, circ)
    final = ref.get_state()
    probs = np.array([[ref.prob(t, o) for o in (0, 1)] for t in range(n)])
    u = uniforms(rng, nshots, False)
    keys, counts = feed_map(ref, u)
    ma_u = uniforms(rng, 1, False)
    copy = oracle.RefQubits("Default", state=final)
    oracle.ref_feed_uniforms(ma_u)
    ma = copy.measure_all()
    return dict(final=final, probs=probs, u=u, keys=keys, counts=counts, measure_all_u=ma_u,
                measure_all=np.uint64(ma), seed=np.int64(seed), layers=np.int32(layers),
                **dict(zip(("names", "q1", "q2", "ang"), encode(circ))))


RESIZE_OPS = ("gate", "add_qubit", "append_qubit", "measure_out", "postselect_out",
              "reallocate", "set_state")


def random_state(rng, n, dt):
    v = rng.uniform(-1, 1, 1 << n) + 1j * rng.uniform(-1, 1, 1 << n)
    return (v / np.linalg.norm(v)).astype(dt)


def case_resize(seed, n0, steps, fp32):
    """The Resize backend through a random script of gates, addQubit,
    appendQubit, measureOut, postselectOut, reallocateState and setState
    with a new size; the state (and the outcome or probability) after
    every step, then every prob and sampleAll.  Step i is RESIZE_OPS[kind[i]]
    with arguments qa[i], qb[i], x[i] (gate: ALL_NAMES[gate[i]] on qa, qb,
    angle x; measure_out: qubit qa, uniform x; postselect_out: qubit qa,
    outcome qb; set_state: a new state of qa qubits, stored in states)."""
    rng = np.random.default_rng(seed)
    dt = np.complex64 if fp32 else np.complex128
    init = random_state(rng, n0, dt)
    ref = oracle.RefQubits("Resize", fp32=fp32, state=init)
    kind, gate, qa, qb, xs, res, states = [], [], [], [], [], [], []
    # The reference's storage: dim_max and the vector's size.  Its
    # reallocateState and setState leave dim_max as it was (resize.cpp:67-98),
    # after which addQubit can write past the vector's end
    # (resize.cpp:111-140); the script adds a qubit only where the
    # reference stays inside its vector.
    dim_max = size = 1 << n0
    for _ in range(steps):
        n = ref.n
        dim = 1 << n
        r = rng.random()
        g, a, b, x, out = -1, 0, -1, 0.0, 0.0
        if 0.4 <= r < 0.68 and not (dim == dim_max or 2 * dim <= size):
            continue
        if r < 0.4:
            k = 0
            g = int(rng.integers(len(ALL_NAMES)))
            a, b = (int(v) for v in rng.choice(n, 2, replace=False))
            if ALL_NAMES[g] in GATES1:
                b = -1
            x = float(rng.uniform(0, 2 * np.pi))
            if fp32:
                x = float(np.float32(x))
            workloads.apply(ref, [(ALL_NAMES[g], a, None if b < 0 else b, x)])
        elif r < 0.68 and n < 10:
            if dim == dim_max:
                size = dim_max = 2 * dim
            if r < 0.62:
                k, a = 1, int(rng.integers(n + 1))
                ref.add_qubit(a)
            else:
                k = 2
                ref.append_qubit()
        elif r < 0.8 and n > 2:
            k, a = 3, int(rng.integers(n))
            x = float(uniforms(rng, 1, fp32)[0])
            oracle.ref_feed_uniforms([x])
            out = float(ref.measure_out(a))
        elif r < 0.92 and n > 2:
            k, a, b = 4, int(rng.integers(n)), int(rng.integers(2))
            if ref.prob(a, b) < 1e-3:
                b ^= 1
            out = float(ref.postselect_out(a, b))
        elif r < 0.96:
            k = 5
            ref.reallocate()
            size = dim
        else:
            k, a = 6, int(rng.integers(2, 10))
            ref.set_state(random_state(rng, a, dt))
            size = 1 << a
        kind.append(k)
        gate.append(g)
        qa.append(a)
        qb.append(b)
        xs.append(x)
        res.append(out)
        states.append(ref.get_state())
    n = ref.n
    probs = np.array([[ref.prob(t, o) for o in (0, 1)] for t in range(n)])
    u = uniforms(rng, 500, fp32)
    keys, counts = feed_map(ref, u)
    return dict(init=init, kind=np.array(kind, dtype=np.int32), gate=np.array(gate, dtype=np.int32),
                qa=np.array(qa, dtype=np.int32), qb=np.array(qb, dtype=np.int32), x=np.array(xs),
                res=np.array(res), state_len=np.array([st.size for st in states], dtype=np.int64),
                states=np.concatenate(states), probs=probs, u=u, keys=keys, counts=counts)


def results_table():
    """A table written by the reference's own Results::writeToFile
    (include/qsl/benchmark/results.tpp:315-355), with values that exercise
    the default float format: tiny, huge, exact, long mantissas."""
    rng = np.random.default_rng(77)
    heads = ["nones", "nqubits", "Default", "Default+OMP", "Cuda", "CudaNP"]
    meta = ["Testing the phase gate", "Results are in seconds"]
    ints = np.array([[w, 16] for w in range(1, 16)], dtype=np.uint32)
    fps = np.concatenate([rng.uniform(1e-6, 1e-4, (15, 2)), 10.0 ** rng.uniform(-9, 9, (15, 2))],
                         axis=1)
    fps[0, :] = [0.1, 1.0, 123456789.0, 1e-7]
    fps[1, :] = [5.11879e-05, 0.0, 100000.0, 999999.5]
    path = os.path.join(HERE, "results_ref.txt")
    rc = oracle.ref_lib().qslref_results_write(path.encode(), "\n".join(heads).encode(),
                                               "\n".join(meta).encode(), 15, 2, ints.ctypes.data, 4,
                                               np.ascontiguousarray(fps).ctypes.data)
    assert rc == 0
    with open(os.path.join(HERE, "results_ref.json"), "w") as f:
        json.dump({"headings": heads, "meta": meta, "ints": ints.tolist(),
                   "fps": [[float(x).hex() for x in row] for row in fps]}, f, indent=0)


def kats():
    lib = oracle.ref_lib()
    seq = [0b111]
    for _ in range(9):
        seq.append(int(lib.qslref_next(seq[-1])))
    lookups = {}
    for length in range(1, 11):
        for ones in range(0, length + 1):
            m = lib.qslref_generate_lookup(length, ones, None, 0)
            out = np.zeros(m, dtype=np.uint64)
            lib.qslref_generate_lookup(length, ones, out.ctypes.data, m)
            lookups[f"{length},{ones}"] = [int(x) for x in out]
    hw = {str(x): int(lib.qslref_hamming_weight(x)) for x in (0b11011010, 0b1010, 0b1, 0)}
    ch = {f"{a},{b}": int(lib.qslref_choose(a, b)) for a, b in ((1, 1), (4, 3), (10, 3), (10, 10), (28, 14))}
    return {"next_from_0b111": seq, "lookups": lookups, "hamming_weight": hw, "choose": ch}


def main():
    oracle.build(reference=True)
    oracle.ref_lib().qslref_seed(12345)
    for fp32 in (False, True):
        tag = "c64" if fp32 else "c128"
        cases = {f"s{s}": case_default(s, 8, fp32) for s in (1, 2, 3)}
        np.savez_compressed(os.path.join(HERE, f"default_{tag}.npz"),
                            **{f"{k}__{f}": v for k, c in cases.items() for f, v in c.items()})
        cases = {"n8w4": case_np(11, 8, 4, fp32), "n10w3": case_np(12, 10, 3, fp32),
                 "n6w1": case_np(13, 6, 1, fp32)}
        np.savez_compressed(os.path.join(HERE, f"np_{tag}.npz"),
                            **{f"{k}__{f}": v for k, c in cases.items() for f, v in c.items()})
    for fp32 in (False, True):
        tag = "c64" if fp32 else "c128"
        cases = {f"r{s}": case_resize(s, 5, 60, fp32) for s in (31, 32, 33)}
        np.savez_compressed(os.path.join(HERE, f"resize_{tag}.npz"),
                            **{f"{k}__{f}": v for k, c in cases.items() for f, v in c.items()})
    lay = case_layered(2021, 12, 20, 10000)
    np.savez_compressed(os.path.join(HERE, "layered_n12.npz"), **lay)
    results_table()
    with open(os.path.join(HERE, "kat.json"), "w") as f:
        json.dump(kats(), f, indent=0, sort_keys=True)
    print("fixtures written to", HERE)


def load_cases(path):
    """{case: {field: array}} from a fixture file written by main()."""
    z = np.load(path)
    out = {}
    for key in z.files:
        case, field = key.split("__", 1)
        out.setdefault(case, {})[field] = z[key]
    return out


if __name__ == "__main__":
    main()
