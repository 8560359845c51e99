"""Gate fusion planner of the precision form (qsl_gb300/csrc/fusion_host.hpp),
on the CPU: gate matrices against the oracle's restatement of the reference
loops, and planned blocks against gate-by-gate application."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_fusion_planner(port, tmp_path):
    exe = os.path.join(str(tmp_path), "fusion_check")
    so = os.path.join(ROOT, "oracle", "libqsl_port.so")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "qsl_gb300", "csrc"),
                        "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle"),
                        os.path.join(ROOT, "tests", "cpp", "fusion_check.cpp"), so,
                        f"-Wl,-rpath,{os.path.dirname(so)}", "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "fusion ok" in r.stdout
