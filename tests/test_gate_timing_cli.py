"""The dense-state gate timer's command line (gate_timing.py, beside
bench.py): argument checks that need no GPU."""
import os

import pytest

import gate_timing


def test_rejects_targets_outside_the_state():
    with pytest.raises(SystemExit):
        gate_timing.main(["--qubits", "10", "--targets", "3,10"])
    with pytest.raises(SystemExit):
        gate_timing.main(["--qubits", "10", "--targets", "-1"])


def test_prepare_dense_touches_every_qubit_twice():
    calls = []

    class Rec:
        def rotateY(self, q, a):
            calls.append(("rotateY", q, a))

        def rotateZ(self, q, a):
            calls.append(("rotateZ", q, a))

    gate_timing.prepare_dense(Rec(), 5)
    assert [c[:2] for c in calls] == [(g, q) for q in range(5) for g in ("rotateY", "rotateZ")]
    assert all(0.3 <= c[2] <= 2.8 for c in calls)


def test_rejects_bad_pairs_and_gates():
    with pytest.raises(SystemExit):
        gate_timing.main(["--qubits", "10", "--pairs", "3:3"])
    with pytest.raises(SystemExit):
        gate_timing.main(["--qubits", "10", "--pairs", "3:10"])
    with pytest.raises(SystemExit):
        gate_timing.main(["--qubits", "10", "--gates", "notAGate"])


def test_algorithmic_bytes_follow_the_reference_loops():
    n = 30
    assert gate_timing.alg_bytes("rotateX", n) == 32 << 30
    assert gate_timing.alg_bytes("phase", n) == 32 << 29
    assert gate_timing.alg_bytes("controlNot", n) == 32 << 29
    assert gate_timing.alg_bytes("controlPhase", n) == 32 << 28


def test_batch_timing_picks_the_bench_instances():
    """batch_timing.py (beside bench.py) runs a sub-batch of the benchmark's
    4096 instances: the first ones plus the largest, ascending."""
    import batch_timing
    idx, (ns, ls, angles, u) = batch_timing.sub_batch(12, 4)
    assert list(idx[:12]) == list(range(12)) and idx.size == 16
    assert np_sorted(idx) and list(ns[-4:]) == [20, 20, 20, 20]
    assert angles.size == int((2 * ns.astype(int) * ls.astype(int)).sum())
    with pytest.raises(SystemExit):
        batch_timing.main(["--first", "0", "--largest", "0"])
    idx, (ns, _, _, _) = batch_timing.sub_batch(300, 0, 14)
    assert idx.size > 0 and int(ns.max()) <= 14 and np_sorted(idx)
    for bad in ("512,12", "512,x,2"):
        with pytest.raises(SystemExit):
            batch_timing.main(["--shape", bad])


def np_sorted(a):
    return all(a[i] < a[i + 1] for i in range(len(a) - 1))


def test_gate_timing_times_single_gates_unless_grouped(monkeypatch):
    """gate_timing.py switches the library's grouping off (each window then
    holds one gate's launch) unless --grouped asks for two gates a window."""
    import gate_timing
    seen = []
    monkeypatch.setattr(gate_timing, "run", lambda *a: seen.append((os.environ.get("QSLC_GROUP"), a[-1])))
    monkeypatch.setenv("QSLC_GROUP", "1")              # restored after the test
    monkeypatch.delenv("QSLC_GROUP")
    gate_timing.main(["--gates", "rotateX", "--targets", "1"])
    assert seen[-1] == ("0", False)
    monkeypatch.delenv("QSLC_GROUP")
    gate_timing.main(["--gates", "rotateX", "--targets", "1", "--grouped"])
    assert seen[-1] == (None, True)
