"""bench.py --gpus N without an outside launcher starts N ranks itself
(bench.launch_ranks, under torch.distributed.run on 127.0.0.1).  On CPU the
launched program is a stand-in with bench.py's rank plumbing -- the
replica layer on `gloo`, the slowest rank's time, one JSON line from rank
0 -- so the test needs no GPU."""
import json
import os
import subprocess
import sys
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STAND_IN = textwrap.dedent("""
    import json, os, sys
    sys.path.insert(0, {root!r})
    from qsl_gb300.replicas import Replicas
    rep = Replicas("gloo")
    with open(os.path.join({out!r}, f"rank{{rep.rank}}.json"), "w") as f:
        json.dump({{k: os.environ.get(k) for k in
                   ("RANK", "LOCAL_RANK", "WORLD_SIZE", "MASTER_ADDR")}}, f)
    seconds = 1.0 + rep.rank
    line = {{"n_gpus": rep.world, "value": rep.throughput(45, seconds),
             "argv": sys.argv[1:]}}
    rep.close()
    if rep.leader:
        print(json.dumps(line), flush=True)
""")


def test_launch_ranks_starts_one_rank_per_gpu(tmp_path):
    pytest.importorskip("torch.distributed")
    sys.path.insert(0, ROOT)
    import bench
    script = tmp_path / "stand_in.py"
    script.write_text(STAND_IN.format(root=ROOT, out=str(tmp_path)))
    log = tmp_path / "out.txt"
    with open(log, "w") as f:
        code = subprocess.call(
            [sys.executable, "-c",
             f"import sys; sys.path.insert(0, {ROOT!r}); import bench; "
             f"sys.exit(bench.launch_ranks(2, ['--steps', '2'], script={str(script)!r}))"],
            stdout=f, stderr=subprocess.STDOUT, timeout=300)
    text = log.read_text()
    assert code == 0, text
    envs = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(2)]
    assert [e["RANK"] for e in envs] == ["0", "1"]
    assert [e["LOCAL_RANK"] for e in envs] == ["0", "1"]
    assert all(e["WORLD_SIZE"] == "2" and e["MASTER_ADDR"] == "127.0.0.1" for e in envs)
    lines = [json.loads(x) for x in text.splitlines() if x.startswith("{")]
    assert len(lines) == 1, text              # rank 0 alone prints
    assert lines[0]["n_gpus"] == 2
    assert lines[0]["value"] == pytest.approx(90 / 2.0)   # both ranks' gates over the slowest time
    assert lines[0]["argv"] == ["--steps", "2"]
    assert bench.free_port() > 0


def test_bench_relaunches_itself_only_without_a_launcher(monkeypatch):
    """With WORLD_SIZE already set (torchrun around it) bench.py does not
    start ranks of its own."""
    sys.path.insert(0, ROOT)
    import bench
    calls = []
    monkeypatch.setattr(bench, "launch_ranks", lambda n, argv, script=None: calls.append(n) or 0)
    monkeypatch.setattr(bench, "run_gpu", lambda args: calls.append("gpu"))
    monkeypatch.setattr(sys, "argv", ["bench.py", "--gpus", "4"])
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    with pytest.raises(SystemExit) as e:
        bench.main()
    assert e.value.code == 0 and calls == [4]
    calls.clear()
    monkeypatch.setenv("WORLD_SIZE", "4")
    bench.main()
    assert calls == ["gpu"]


def test_launch_windows_follow_the_grouping():
    """The bench's timing windows mirror the library's grouping: a held
    one-qubit gate joins the next one on another qubit, is released alone
    by a gate on the same qubit, and by an explicit flush before a
    two-qubit gate and at the end of a layer."""
    import bench
    ry0, rz1, h2, p2, h3 = (("rotateY", 0, None, .1), ("rotateZ", 1, None, .2), ("hadamard", 2, None, 0.),
                            ("phase", 2, None, .3), ("hadamard", 3, None, 0.))
    cx = ("controlNot", 0, 1, 0.)
    w = bench.launch_windows([ry0, rz1, h2, p2, cx, h3])
    assert w == [(ry0, None), (rz1, [ry0, rz1]), (h2, None), (p2, [h2]), (None, [p2]), (cx, [cx]),
                 (h3, None), (None, [h3])]
    assert bench.launch_windows([ry0, rz1], grouping=False) == [(ry0, [ry0]), (rz1, [rz1])]
    launched = [g for _, gs in w if gs for g in gs]
    assert launched == [ry0, rz1, h2, p2, cx, h3]
