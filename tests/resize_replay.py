"""Replays a Resize fixture script (tests/golden/make_golden.py case_resize)
on a simulator and checks every step against the reference's recorded
states, outcomes and probabilities, bit for bit.

``ops`` adapts the simulator: a dict of callables add_qubit(t),
append_qubit(), measure_out(t, u), postselect_out(t, o), reallocate(),
set_state(state), gate(name, q1, q2, angle), get_state(), prob(t, o),
sample_all(u) -> per-shot indices."""
import numpy as np

from conftest import bits
from golden.make_golden import ALL_NAMES, GATES1, RESIZE_OPS


def replay(case, ops, dtype, exact=True):
    """``exact=False`` (complex64 gates, whose host-side float cos/sin may
    round differently from the reference's libm): a state that differs from
    the reference's is held to 1e-5 and replaced by the reference's bits
    before the next step, so every later step starts from the same input."""
    rdt = np.float32 if dtype == np.complex64 else np.float64
    offs = np.concatenate([[0], np.cumsum(case["state_len"])])
    for i, k in enumerate(case["kind"]):
        name = RESIZE_OPS[int(k)]
        a, b, x = int(case["qa"][i]), int(case["qb"][i]), float(case["x"][i])
        want = case["states"][offs[i]:offs[i + 1]]
        if name == "gate":
            g = ALL_NAMES[int(case["gate"][i])]
            ops["gate"](g, a, None if g in GATES1 else b, x)
        elif name == "add_qubit":
            ops["add_qubit"](a)
        elif name == "append_qubit":
            ops["append_qubit"]()
        elif name == "measure_out":
            assert ops["measure_out"](a, x) == int(case["res"][i]), f"step {i}: measureOut outcome"
        elif name == "postselect_out":
            p = ops["postselect_out"](a, b)
            assert rdt(p) == rdt(case["res"][i]), f"step {i}: postselectOut probability"
        elif name == "reallocate":
            ops["reallocate"]()
        elif name == "set_state":
            ops["set_state"](want)
        got = ops["get_state"]()
        want = want.astype(dtype)
        assert got.size == want.size, f"step {i} ({name}): {got.size} amplitudes, want {want.size}"
        if not np.array_equal(bits(got), bits(want)):
            assert not exact, f"step {i} ({name})"
            assert np.abs(got - want).max() <= 1e-5, f"step {i} ({name})"
            ops["set_state"](want)
    n = int(np.log2(case["state_len"][-1]))
    probs = np.array([[ops["prob"](t, o) for o in (0, 1)] for t in range(n)], dtype=rdt)
    assert np.array_equal(probs, case["probs"].astype(rdt))
    k, c = np.unique(ops["sample_all"](case["u"]), return_counts=True)
    assert np.array_equal(k, case["keys"]) and np.array_equal(c, case["counts"])
