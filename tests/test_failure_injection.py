"""Failure handling, tested from the host with no GPU fault.

The C ABI turns every failure into a status and a message: a bad argument
(QSLC_EINVAL, where the reference's behaviour is undefined or it throws
std::logic_error, default.cpp:70-74), a failed device allocation
(QSLC_EOOM), a CUDA runtime error (QSLC_ECUDA).  The Python mirror raises
LogicError / QslcError for them, and the C++ drop-in std::logic_error /
std::runtime_error.  Failures are made on the host: QSLC_FORCE_ERROR makes
an entry point fail (read when the library loads, so each case runs in a
child process), an allocation too large for any GPU fails for real, and on
a machine without a GPU every state creation fails.  Nothing here faults,
traps or hangs a device."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "tests", "cpp")


def run_py(code: str, force: str | None = None) -> dict:
    """Run `code` (which prints one JSON line) in a child process, with
    QSLC_FORCE_ERROR set to `force`."""
    env = dict(os.environ)
    env.pop("QSLC_FORCE_ERROR", None)
    if force is not None:
        env["QSLC_FORCE_ERROR"] = force
    prog = f"import sys, json, ctypes as C; sys.path.insert(0, {ROOT!r}); import qsl_gb300 as q\n" + code
    r = subprocess.run([sys.executable, "-c", prog], capture_output=True, text=True, env=env,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout.strip().splitlines()[-1])


def build_error_map(qsl, tmp):
    exe = os.path.join(tmp, "error_map")
    libdir = os.path.dirname(qsl.LIB_PATH)
    r = subprocess.run(["g++", "-std=c++20", "-O1", "-I", os.path.join(ROOT, "include"),
                        os.path.join(CPP, "error_map.cpp"), "-o", exe, "-L", libdir, "-lqslc",
                        f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def run_error_map(exe, n, force=None) -> str:
    env = dict(os.environ)
    env.pop("QSLC_FORCE_ERROR", None)
    if force is not None:
        env["QSLC_FORCE_ERROR"] = force
    r = subprocess.run([exe, str(n)], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr
    return r.stdout.strip()


CREATE = """
h = C.c_void_p()
L = q.lib()
rc = L.qslc_create(6, q.C128, C.byref(h))
print(json.dumps({"rc": rc, "msg": L.qslc_last_error().decode()}))
"""


@pytest.mark.parametrize("code", [1, 2, 3, 4, 6])
def test_forced_status_reaches_the_caller(qsl, code):
    out = run_py(CREATE, force=f"qslc_create:{code}")
    assert out["rc"] == code
    assert out["msg"] == "forced failure of qslc_create (QSLC_FORCE_ERROR)"


def test_forced_error_defaults_to_a_cuda_error_and_matches_by_name(qsl):
    assert run_py(CREATE, force="qslc_create")["rc"] == qsl.ECUDA
    assert run_py(CREATE, force="*:2")["rc"] == qsl.EOOM
    # another entry point's name leaves qslc_create alone (it then fails
    # only if there is no GPU, and not with the forced message)
    out = run_py(CREATE, force="qslc_gate1:2")
    assert "QSLC_FORCE_ERROR" not in out["msg"]


def test_forced_error_after_some_successful_calls(qsl):
    """name:code:after -- the first `after` calls run normally (here they
    fail on the null handle, as unforced calls do), the next ones are
    forced."""
    out = run_py("""
L = q.lib()
rcs, msgs = [], []
for _ in range(4):
    rcs.append(L.qslc_gate1(None, q.GATE1["rotateX"], 0, 0.1))
    msgs.append(L.qslc_last_error().decode())
print(json.dumps({"rcs": rcs, "msgs": msgs}))
""", force="qslc_gate1:4:2")
    assert out["rcs"] == [qsl.EINVAL, qsl.EINVAL, qsl.ETIMEOUT, qsl.ETIMEOUT]
    assert "null" in out["msgs"][0] and "QSLC_FORCE_ERROR" in out["msgs"][2]


def test_python_mirror_maps_status_to_exceptions(qsl):
    prog = """
try:
    q.Qubits(6)
    res = "ok"
except q.LogicError as e:
    res = ["LogicError", e.code]
except q.QslcError as e:
    res = ["QslcError", e.code]
print(json.dumps(res))
"""
    assert run_py(prog, force="qslc_create:2") == ["QslcError", qsl.EOOM]
    assert run_py(prog, force="qslc_create:3") == ["QslcError", qsl.ECUDA]
    assert run_py(prog, force="qslc_create:6") == ["LogicError", qsl.ESIZE]
    assert run_py(prog, force="qslc_create:1") == ["LogicError", qsl.EINVAL]


def test_cpp_drop_in_maps_status_to_exceptions(qsl, tmp_path):
    """std::runtime_error for allocation and CUDA failures, std::logic_error
    where the reference throws it (a size mismatch, a bad argument)."""
    exe = build_error_map(qsl, str(tmp_path))
    assert run_error_map(exe, 6, "qslc_create:2") == \
        "runtime_error: forced failure of qslc_create (QSLC_FORCE_ERROR)"
    assert run_error_map(exe, 6, "qslc_create:3").startswith("runtime_error: forced")
    assert run_error_map(exe, 6, "qslc_create:6") == \
        "logic_error: forced failure of qslc_create (QSLC_FORCE_ERROR)"
    assert run_error_map(exe, 6, "qslc_create:1").startswith("logic_error: forced")


def test_no_gpu_means_a_loud_failure(qsl, tmp_path):
    """Where CUDA sees no device, creating a state fails with a CUDA error
    and a message -- there is no CPU fallback to fall into."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    out = run_py(CREATE)
    assert out["rc"] == qsl.ECUDA and "CUDA error" in out["msg"]
    exe = build_error_map(qsl, str(tmp_path))
    assert run_error_map(exe, 6).startswith("runtime_error: CUDA error")


@pytest.mark.gpu
def test_impossible_allocation_is_out_of_memory(qsl, tmp_path):
    """40 qubits of complex128 (16 TiB) cannot be allocated: QSLC_EOOM with
    the size in the message, QslcError in Python, std::runtime_error in C++;
    the library stays usable afterwards."""
    with pytest.raises(qsl.QslcError) as e:
        qsl.Qubits(40)
    assert e.value.code == qsl.EOOM and "17592186044416 bytes" in str(e.value)
    with pytest.raises(qsl.QslcError) as e:
        qsl.Qubits(39, dtype=np.complex64)
    assert e.value.code == qsl.EOOM
    ok = qsl.Qubits(8)
    ok.hadamard(3)
    assert abs(ok.prob(3, 1) - 0.5) <= 1e-15
    exe = build_error_map(qsl, str(tmp_path))
    out = run_error_map(exe, 40)
    assert out.startswith("runtime_error: out of device memory"), out
    assert run_error_map(exe, 10).startswith("ok ")


@pytest.mark.gpu
def test_failure_mid_circuit_leaves_the_state_usable(qsl, port):
    """The sixth gate call is forced to fail: the five before it are applied,
    the handle answers afterwards, and its state is the oracle's after those
    five gates."""
    out = run_py("""
import numpy as np
s = q.Qubits(10)
gates = [("hadamard", 0), ("rotateX", 3), ("rotateY", 9), ("phase", 2), ("rotateZ", 5),
         ("rotateX", 1), ("hadamard", 7)]
done, err = 0, None
for g, t in gates:
    try:
        s.gate(g, t, None, 0.37)
        done += 1
    except q.QslcError as e:
        err = [e.code, str(e)]
        break
st = s.getState()
print(json.dumps({"done": done, "err": err, "p": s.prob(0, 1),
                  "state": [st.real.tolist(), st.imag.tolist()]}))
""", force="qslc_gate1:3:5")
    assert out["done"] == 5 and out["err"][0] == qsl.ECUDA
    cpu = port.PortQubits(10)
    for g, t in [("hadamard", 0), ("rotateX", 3), ("rotateY", 9), ("phase", 2), ("rotateZ", 5)]:
        cpu.gate(g, t, None, 0.37)
    got = np.array(out["state"][0]) + 1j * np.array(out["state"][1])
    assert np.array_equal(got, cpu.state)
    assert out["p"] == cpu.prob(0, 1)
