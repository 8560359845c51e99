"""The integer-pipe binary64 multiply/add (qsl_gb300/csrc/dpemu.cuh) equals
the host's IEEE round-to-nearest arithmetic bit for bit, on millions of
operands chosen to hit exact results, rounding ties, cancellation, large
exponent gaps, zeros and the overflow/underflow edges."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_dpemu_matches_ieee(tmp_path):
    exe = os.path.join(str(tmp_path), "dpemu_check")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I",
                        os.path.join(ROOT, "qsl_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "cpp", "dpemu_check.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "4000000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "dpemu ok" in r.stdout
