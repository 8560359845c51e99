"""Host-side NP index arithmetic (Gosper stepping, rank/unrank, scatter and
gather of the compressed layout) checked exhaustively on the CPU."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_np_host_index_arithmetic(tmp_path):
    exe = os.path.join(str(tmp_path), "np_host_check")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "qsl_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "cpp", "np_host_check.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr + r.stdout
    assert "np_host ok" in r.stdout
