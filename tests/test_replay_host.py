"""The exact replay of a sequential floating-point sum (replay.cuh), checked
on the CPU against the sequential loop itself: runs of terms composed as
parity transducers in one binade give the sequentially rounded sum,
including exact ties (float terms in a double sum, repeated terms)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_replay_matches_sequential_sum(tmp_path):
    exe = os.path.join(str(tmp_path), "replay_check")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I",
                        os.path.join(ROOT, "qsl_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "cpp", "replay_check.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "replay ok" in r.stdout
