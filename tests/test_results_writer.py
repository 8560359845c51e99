"""qsl's Results table (include/qsl/benchmark/results.hpp:49-246), restated
in qsl_gb300/results.py: the file it writes is byte for byte the one the
reference's own writeToFile wrote for the same table
(tests/golden/results_ref.txt), and the statistics follow results.tpp."""
import json
import math
import os

import numpy as np
import pytest

from qsl_gb300.results import Results

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def table():
    spec = json.load(open(os.path.join(GOLD, "results_ref.json")))
    r = Results(spec["headings"])
    for m in spec["meta"]:
        r.addMeta(m)
    for ints, fps in zip(spec["ints"], spec["fps"]):
        r.addRow(ints, [float.fromhex(x) for x in fps])
    return r


def test_write_matches_reference_bytes(tmp_path):
    out = tmp_path / "t.csv"
    table().writeToFile(str(out))
    assert out.read_bytes() == open(os.path.join(GOLD, "results_ref.txt"), "rb").read()


def test_file_reads_back_as_columns(tmp_path):
    """The layout qsl's scripts/plot.py reads: '#' comments, then a header
    row and whitespace-separated columns."""
    out = tmp_path / "t.csv"
    r = table()
    r.writeToFile(str(out))
    lines = [ln.split("#")[0].split() for ln in open(out)]
    lines = [ln for ln in lines if ln]
    head, rows = lines[0], np.array(lines[1:], dtype=float)
    assert head == ["nones", "nqubits", "Default", "Default+OMP", "Cuda", "CudaNP"]
    assert rows[:, 0].tolist() == list(range(1, 16))
    assert np.allclose(rows[:, 4], r.column("Cuda"), rtol=1e-5)


def test_statistics_and_errors():
    r = table()
    col = r.column("Default")
    assert r.mean("Default") == pytest.approx(sum(col) / len(col))
    m = sum(col) / len(col)
    assert r.variance(2) == pytest.approx(sum((x - m) ** 2 for x in col) / (len(col) - 1))
    assert r.mean("nones") == 8.0
    s = r.subset(["CudaNP", "nones"])
    assert s.headings() == ["CudaNP", "nones"]
    # the reference stores a subset's integer columns first whatever the
    # order asked for (results.tpp:236-262), so position 0 reads "nones"
    assert s.column(0) == list(range(1, 16))
    assert s.intcols[0] == [1] and s.fpcols[0] == [r.fpcols[0][3]]
    with pytest.raises(ValueError):
        r.addRow([1], [1.0, 2.0, 3.0, 4.0])            # wrong integer column count
    with pytest.raises(ValueError):
        r.mean("missing")
    with pytest.raises(IndexError):
        r.mean(6)
    e = Results(["a", "b"])
    with pytest.raises(ValueError):
        e.addRow([1, 2], [3.0])                         # 3 values, 2 headings
    assert math.isnan(e.mean(0)) and e.variance(0) == 0.0 and e.column(1) == []


@pytest.mark.gpu
def test_np_phase_benchmark_writes_reference_format(qsl, tmp_path):
    """qsl's examples/benchmark-np.cpp on the GPU, small: one row per
    number of ones, positive times, the reference's file layout."""
    from qsl_gb300 import benchmark_np
    out = tmp_path / "np_phase_cuda.csv"
    benchmark_np.main(["--nqubits", "8", "--reps", "20", "--out", str(out)])
    text = out.read_text().splitlines()
    assert text[0] == "# Testing the phase gate" and text[1] == "" and text[2] == "nones Cuda CudaNP"
    rows = np.array([ln.split() for ln in text[3:]], dtype=float)
    assert rows[:, 0].tolist() == list(range(1, 8))
    assert np.all(rows[:, 1:] > 0) and np.all(rows[:, 1:] < 1)
