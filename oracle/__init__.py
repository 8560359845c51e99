"""The oracle: CPU restatement of qsl's hot path, and the reference itself.

TEST INFRASTRUCTURE ONLY.  Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this package, and only as the checker
or as the timed CPU baseline.  The CUDA backend (``qsl_gb300``) never imports
it.

Two libraries sit behind it:

* ``libqsl_port.so`` (``qsl_port.c``): a plain-C restatement of the
  reference's Default / OpenMP / NP loops (src/qubits/default/*.cpp,
  src/qubits/np/*.cpp, src/utils/misc.cpp).  It builds on any host.
* ``_ref/libqslref.so``: the reference's own sources, compiled unmodified
  with a seedable replacement for src/utils/random.cpp.  It is only built
  where the reference source tree is present; tests/golden holds what it
  produced so the restatement stays pinned where it is absent.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "libqsl_port.so")
REF_SO = os.path.join(HERE, "_ref", "libqslref.so")


def _ref_src() -> str:
    """The reference's source tree: QSL_REFERENCE_SRC, else the default that
    oracle/Makefile holds (asked for with `make -s print-ref`)."""
    env = os.environ.get("QSL_REFERENCE_SRC")
    if env:
        return env
    try:
        out = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True,
                             text=True, timeout=60)
        return out.stdout.strip() if out.returncode == 0 else ""
    except (OSError, subprocess.SubprocessError):
        return ""


REF_SRC = _ref_src()

ONE_QUBIT = ("pauliX", "pauliY", "pauliZ", "hadamard", "phase", "rotateX", "rotateY", "rotateZ")
ANGLED = {"phase", "rotateX", "rotateY", "rotateZ", "controlRotateX", "controlRotateY",
          "controlRotateZ", "controlPhase", "npRotateX", "npRotateY"}
TWO_QUBIT = ("controlNot", "controlY", "controlZ", "controlRotateX", "controlRotateY",
             "controlRotateZ", "controlPhase", "controlHadamard", "swap", "fswap",
             "npRotateX", "npRotateY", "npHadamard")
NP_GATES = ("pauliZ", "rotateZ", "phase", "controlZ", "controlRotateZ", "controlPhase",
            "swap", "fswap", "npRotateX", "npRotateY", "npHadamard")

# op codes of port_*_gate2 / port_*_np_gate2 (oracle/qsl_port.h)
_OP2 = {g: i for i, g in enumerate(("controlNot", "controlY", "controlZ", "controlRotateX",
                                    "controlRotateY", "controlRotateZ", "controlPhase",
                                    "controlHadamard", "swap", "fswap", "npRotateX",
                                    "npRotateY", "npHadamard"))}
_NP2 = {"controlZ": 0, "controlPhase": 1, "crz01": 2, "swap": 3, "npRotateX": 4,
        "npRotateY": 5, "npHadamard": 6}


def build(reference: bool | None = None, quiet: bool = True) -> None:
    """Build the restatement, and the reference library when its sources exist."""
    targets = ["port"]
    if reference is None:
        reference = bool(REF_SRC) and os.path.isdir(os.path.join(REF_SRC, "src", "qubits"))
    if reference:
        targets.append("ref")
    jobs = str(max(1, min(16, os.cpu_count() or 1)))
    out = subprocess.run(["make", "-C", HERE, "-j", jobs, f"REF={REF_SRC}", *targets],
                         capture_output=quiet, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{out.stdout}\n{out.stderr}")


def ref_available() -> bool:
    return os.path.exists(REF_SO)


_port = None
_ref = None

_u64p = C.POINTER(C.c_uint64)
_dblp = C.POINTER(C.c_double)


def port_lib():
    global _port
    if _port is None:
        if not os.path.exists(PORT_SO):
            build(reference=False)
        lib = C.CDLL(PORT_SO)
        for sfx, fp in (("d", C.c_double), ("f", C.c_float)):
            vp = C.c_void_p
            def sig(name, res, *args):
                f = getattr(lib, f"port_{sfx}_{name}")
                f.restype = res
                f.argtypes = list(args)
            for g in ("pauliX", "pauliY", "pauliZ", "hadamard"):
                sig(g, None, vp, C.c_uint, C.c_uint, C.c_int)
            for g in ("phase", "rotateX", "rotateY", "rotateZ"):
                sig(g, None, vp, C.c_uint, C.c_uint, fp, C.c_int)
            sig("gate2", None, vp, C.c_uint, C.c_int, C.c_uint, C.c_uint, fp, C.c_int)
            sig("prob", fp, vp, C.c_uint, C.c_uint, C.c_uint)
            sig("prob_omp", fp, vp, C.c_uint, C.c_uint, C.c_uint, C.c_int)
            sig("collapse", None, vp, C.c_uint, C.c_uint, C.c_uint, fp, C.c_int)
            sig("measure", C.c_int, vp, C.c_uint, C.c_uint, fp)
            sig("postselect", fp, vp, C.c_uint, C.c_uint, C.c_uint)
            sig("generate_dist", C.c_size_t, vp, C.c_uint, vp, vp)
            sig("draw_sample", C.c_uint64, vp, vp, C.c_size_t, fp)
            sig("measure_all", C.c_uint64, vp, C.c_uint, fp, vp, vp)
            sig("sample_all", None, vp, C.c_uint, vp, C.c_size_t, vp, vp, vp)
            sig("sample", None, vp, C.c_uint, C.c_uint, vp, C.c_size_t, vp)
            sig("sample_all2", None, vp, C.c_uint, vp, C.c_size_t, vp)
            sig("add_qubit", None, vp, C.c_uint, C.c_uint)
            sig("collapse_out", None, vp, C.c_uint, C.c_uint, C.c_uint, fp)
            sig("np_phase1", None, vp, vp, C.c_size_t, C.c_uint, C.c_int, fp, C.c_int)
            sig("np_rz0", None, vp, vp, C.c_size_t, C.c_uint, fp, C.c_int)
            sig("np_gate2", None, vp, vp, C.c_size_t, C.c_int, C.c_uint, C.c_uint, fp, C.c_int)
            sig("np_prob", fp, vp, vp, C.c_size_t, C.c_uint, C.c_uint)
            sig("np_collapse", None, vp, vp, C.c_size_t, vp, C.c_size_t, C.c_uint, C.c_uint, fp)
            sig("np_generate_dist", C.c_size_t, vp, vp, C.c_size_t, vp, vp)
            sig("np_sample_all2", None, vp, vp, C.c_size_t, vp, C.c_size_t, vp)
        lib.port_next.restype = C.c_uint64
        lib.port_next.argtypes = [C.c_uint64]
        lib.port_hamming_weight.restype = C.c_uint
        lib.port_hamming_weight.argtypes = [C.c_uint64]
        lib.port_choose.restype = C.c_uint
        lib.port_choose.argtypes = [C.c_uint, C.c_uint]
        lib.port_generate_lookup.restype = C.c_size_t
        lib.port_generate_lookup.argtypes = [C.c_uint, C.c_uint, C.c_void_p, C.c_size_t]
        lib.port_check_state_np_d.restype = C.c_int
        lib.port_check_state_np_d.argtypes = [C.c_void_p, C.c_uint]
        lib.port_num_threads.restype = C.c_int
        _port = lib
    return _port


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def generate_lookup(length: int, ones: int) -> np.ndarray:
    """misc.cpp:75-90: ascending integers with `ones` set bits in `length` bits."""
    lib = port_lib()
    m = lib.port_generate_lookup(length, ones, None, 0)
    out = np.empty(m, dtype=np.uint64)
    lib.port_generate_lookup(length, ones, _ptr(out), m)
    return out


def next_bits(x: int) -> int:
    return int(port_lib().port_next(x))


class PortQubits:
    """Default / Omp backend restatement on a host array (complex128 or complex64).

    Gates and measurement follow src/qubits/default/{gates,measure}.cpp; the
    uniforms that the reference draws from ``random.getNum()`` are passed in.
    ``nthreads > 1`` runs the sweeps as the Omp backend parallelises them.
    """

    def __init__(self, nqubits: int, fp32: bool = False, nthreads: int = 1, state=None):
        self.n = nqubits
        self.fp32 = fp32
        self.dtype = np.complex64 if fp32 else np.complex128
        self.rdtype = np.float32 if fp32 else np.float64
        self.nth = nthreads
        self.sfx = "f" if fp32 else "d"
        self.lib = port_lib()
        if state is None:
            self.state = np.zeros(1 << nqubits, dtype=self.dtype)
            self.state[0] = 1
        else:
            self.state = np.ascontiguousarray(state, dtype=self.dtype).copy()
            assert self.state.size == 1 << nqubits

    def _f(self, name):
        return getattr(self.lib, f"port_{self.sfx}_{name}")

    def gate(self, name: str, q1: int, q2: int | None = None, angle: float = 0.0) -> None:
        p = _ptr(self.state)
        if name in ONE_QUBIT:
            if name in ANGLED:
                self._f(name)(p, self.n, q1, self.rdtype(angle), self.nth)
            else:
                self._f(name)(p, self.n, q1, self.nth)
        else:
            self._f("gate2")(p, self.n, _OP2[name], q1, q2, self.rdtype(angle), self.nth)

    def prob(self, targ: int, outcome: int) -> float:
        return float(self._f("prob")(_ptr(self.state), self.n, targ, outcome))

    def collapse(self, targ, outcome, factor):
        self._f("collapse")(_ptr(self.state), self.n, targ, outcome, self.rdtype(factor), self.nth)

    def measure(self, targ: int, u: float) -> int:
        return int(self._f("measure")(_ptr(self.state), self.n, targ, self.rdtype(u)))

    def postselect(self, targ: int, outcome: int) -> float:
        return float(self._f("postselect")(_ptr(self.state), self.n, targ, outcome))

    def _scratch(self):
        m = 1 << self.n
        return np.empty(m, dtype=np.uint64), np.empty(m, dtype=np.float64)

    def dist(self):
        idx, cdf = self._scratch()
        m = self._f("generate_dist")(_ptr(self.state), self.n, _ptr(idx), _ptr(cdf))
        return idx[:m].copy(), cdf[:m].copy()

    def measure_all(self, u: float) -> int:
        idx, cdf = self._scratch()
        return int(self._f("measure_all")(_ptr(self.state), self.n, self.rdtype(u),
                                          _ptr(idx), _ptr(cdf)))

    def sample_all(self, uniforms) -> np.ndarray:
        u = np.ascontiguousarray(uniforms, dtype=self.rdtype)
        out = np.empty(u.size, dtype=np.uint64)
        idx, cdf = self._scratch()
        self._f("sample_all")(_ptr(self.state), self.n, _ptr(u), u.size, _ptr(out),
                              _ptr(idx), _ptr(cdf))
        return out

    def sample(self, targ: int, uniforms) -> np.ndarray:
        u = np.ascontiguousarray(uniforms, dtype=self.rdtype)
        counts = np.zeros(2, dtype=np.uint64)
        self._f("sample")(_ptr(self.state), self.n, targ, _ptr(u), u.size, _ptr(counts))
        return counts

    def sample_all2(self, uniforms) -> np.ndarray:
        u = np.sort(np.ascontiguousarray(uniforms, dtype=self.rdtype))
        counts = np.zeros(1 << self.n, dtype=np.uint64)
        self._f("sample_all2")(_ptr(self.state), self.n, _ptr(u), u.size, _ptr(counts))
        return counts


class PortResizeQubits(PortQubits):
    """Resize backend restatement (src/qubits/resize/*.cpp): the Default
    arithmetic on a state whose qubit count changes.  ``cap`` mirrors the
    reference's dim_max: the storage doubles when a qubit is added to a full
    vector, and is kept when one is removed."""

    def __init__(self, nqubits: int, fp32: bool = False, state=None):
        super().__init__(nqubits, fp32=fp32, state=state)
        self.buf = self.state
        self.cap = self.state.size

    def _live(self):
        self.state = self.buf[: 1 << self.n]

    def set_state(self, st) -> None:
        """resize.cpp:67-78: any power-of-two size"""
        st = np.ascontiguousarray(st, dtype=self.dtype)
        m = st.size
        if m < 1 or m & (m - 1):
            raise ValueError("State vector size is not a power of two")
        if m > self.cap:
            self.buf = np.zeros(m, dtype=self.dtype)
            self.cap = m
        self.buf[:m] = st
        self.n = m.bit_length() - 1
        self._live()

    def add_qubit(self, targ: int) -> None:
        """resize.cpp:106-147"""
        dim = 1 << self.n
        if dim == self.cap:
            grown = np.zeros(2 * dim, dtype=self.dtype)
            grown[:dim] = self.buf[:dim]
            self.buf, self.cap = grown, 2 * dim
        self._f("add_qubit")(_ptr(self.buf), self.n, targ)
        self.n += 1
        self._live()

    def append_qubit(self) -> None:
        """resize.cpp:100-104"""
        self.add_qubit(self.n)

    def collapse_out(self, targ: int, outcome: int, factor) -> None:
        self._f("collapse_out")(_ptr(self.buf), self.n, targ, outcome, self.rdtype(factor))
        self.n -= 1
        self._live()

    def measure_out(self, targ: int, u: float) -> int:
        """resize/measure.cpp:156-182"""
        p0 = self.rdtype(self.prob(targ, 0))
        u = self.rdtype(u)
        one = self.rdtype(1)
        if u < p0:
            outcome, factor = 0, one / np.sqrt(p0)
        else:
            outcome, factor = 1, one / np.sqrt(one - p0)
        self.collapse_out(targ, outcome, factor)
        return outcome

    def postselect_out(self, targ: int, outcome: int) -> float:
        """resize/measure.cpp:238-251"""
        p = self.rdtype(self.prob(targ, outcome))
        self.collapse_out(targ, outcome, self.rdtype(1) / np.sqrt(p))
        return float(p)

    def reallocate(self) -> None:
        """resize.cpp:92-98"""
        self.buf = self.buf[: 1 << self.n].copy()
        self.cap = self.buf.size
        self._live()


class PortNPQubits:
    """NP backend restatement (src/qubits/np/*.cpp): full 2^n state and the five
    lookup tables of np.cpp:168-181."""

    def __init__(self, nqubits: int, nones: int = 1, fp32: bool = False, nthreads: int = 1,
                 state=None):
        if not (1 <= nones < nqubits):
            raise ValueError("The number of ones must be 1 <= nones < nqubits.")
        self.n = nqubits
        self.fp32 = fp32
        self.dtype = np.complex64 if fp32 else np.complex128
        self.rdtype = np.float32 if fp32 else np.float64
        self.nth = nthreads
        self.sfx = "f" if fp32 else "d"
        self.lib = port_lib()
        self.set_num_ones(nones, reset=state is None)
        if state is not None:
            self.state = np.ascontiguousarray(state, dtype=self.dtype).copy()

    def set_num_ones(self, w: int, reset: bool = True) -> None:
        n = self.n
        self.w = w
        self.tab = {}
        for key in ((n - 1, w - 1), (n - 2, w - 1), (n - 2, w - 2), (n - 1, w), (n, w)):
            if key[1] >= 0:
                self.tab[key] = generate_lookup(*key)
        if reset:
            self.state = np.zeros(1 << n, dtype=self.dtype)
            self.state[(1 << w) - 1] = 1

    def _f(self, name):
        return getattr(self.lib, f"port_{self.sfx}_{name}")

    def _t(self, length, ones):
        t = self.tab[(length, ones)]
        return _ptr(t), t.size

    def gate(self, name: str, q1: int, q2: int | None = None, angle: float = 0.0) -> None:
        n, w, p, th = self.n, self.w, _ptr(self.state), self.nth
        a = self.rdtype(angle)
        half = self.rdtype(a / self.rdtype(2))
        if name == "phase":
            self._f("np_phase1")(p, *self._t(n - 1, w - 1), q1, 0, a, th)
        elif name == "pauliZ":
            self._f("np_phase1")(p, *self._t(n - 1, w - 1), q1, 1, a, th)
        elif name == "rotateZ":
            self._f("np_rz0")(p, *self._t(n - 1, w), q1, a, th)
            self._f("np_phase1")(p, *self._t(n - 1, w - 1), q1, 0, half, th)
        elif name in ("controlZ", "controlPhase"):
            if w >= 2:
                self._f("np_gate2")(p, *self._t(n - 2, w - 2), _NP2[name], q1, q2, a, th)
        elif name == "controlRotateZ":
            self._f("np_gate2")(p, *self._t(n - 2, w - 1), _NP2["crz01"], q1, q2, a, th)
            if w >= 2:
                self._f("np_gate2")(p, *self._t(n - 2, w - 2), _NP2["controlPhase"], q1, q2,
                                    half, th)
        elif name == "fswap":
            self.gate("swap", q1, q2)
            self.gate("controlZ", q1, q2)
        elif name in ("swap", "npRotateX", "npRotateY", "npHadamard"):
            self._f("np_gate2")(p, *self._t(n - 2, w - 1), _NP2[name], q1, q2, a, th)
        else:
            raise ValueError(f"{name} is not a number-preserving gate")

    def prob(self, targ: int, outcome: int) -> float:
        return float(self._f("np_prob")(_ptr(self.state), *self._t(self.n - 1, self.w - outcome),
                                        targ, outcome))

    def collapse(self, targ, outcome, factor):
        n, w = self.n, self.w
        self._f("np_collapse")(_ptr(self.state), *self._t(n - 1, w - outcome),
                               *self._t(n - 1, w - (outcome ^ 1)), targ, outcome,
                               self.rdtype(factor))

    def measure(self, targ: int, u: float) -> int:
        p0 = self.rdtype(self.prob(targ, 0))
        u = self.rdtype(u)
        one = self.rdtype(1)
        if u < p0:
            outcome, factor = 0, one / np.sqrt(p0)
        else:
            outcome, factor = 1, one / np.sqrt(one - p0)
        self.collapse(targ, outcome, factor)
        return outcome

    def postselect(self, targ: int, outcome: int) -> float:
        p = self.rdtype(self.prob(targ, outcome))
        self.collapse(targ, outcome, self.rdtype(1) / np.sqrt(p))
        return float(p)

    def dist(self):
        t, m = self._t(self.n, self.w)
        idx = np.empty(m, dtype=np.uint64)
        cdf = np.empty(m, dtype=np.float64)
        k = self._f("np_generate_dist")(_ptr(self.state), t, m, _ptr(idx), _ptr(cdf))
        return idx[:k].copy(), cdf[:k].copy()

    def sample_all(self, uniforms) -> np.ndarray:
        u = np.ascontiguousarray(uniforms, dtype=self.rdtype)
        idx, cdf = self.dist()
        f = self._f("draw_sample")
        return np.array([f(_ptr(idx), _ptr(cdf), idx.size, x) for x in u], dtype=np.uint64)

    def sample_all2(self, uniforms) -> np.ndarray:
        """counts per weight-w basis index (table {n, w} order)"""
        u = np.sort(np.ascontiguousarray(uniforms, dtype=self.rdtype))
        t, m = self._t(self.n, self.w)
        counts = np.zeros(m, dtype=np.uint64)
        self._f("np_sample_all2")(_ptr(self.state), t, m, _ptr(u), u.size, _ptr(counts))
        return counts

    def measure_all(self, u: float) -> int:
        out = int(self.sample_all([u])[0])
        self.state[:] = 0
        self.state[out] = 1
        return out


class RefQubits:
    """The reference's own qsl::Qubits<Type, Fp> (oracle/_ref/libqslref.so)."""

    KINDS = {"Default": 0, "Omp": 1, "NP": 2, "OmpNP": 3, "Resize": 4}

    def __init__(self, kind: str, nqubits: int = 0, nones: int = 1, fp32: bool = False,
                 nthreads: int = 1, state=None, seed: int | None = None):
        lib = ref_lib()
        if seed is not None:
            lib.qslref_seed(seed)
        self.lib = lib
        self.fp32 = fp32
        self.dtype = np.complex64 if fp32 else np.complex128
        if state is None:
            h = lib.qslref_create(self.KINDS[kind], int(fp32), nqubits, nones, nthreads)
        else:
            st = np.ascontiguousarray(state, dtype=self.dtype)
            h = lib.qslref_create_from_state(self.KINDS[kind], int(fp32), _ptr(st), st.size,
                                             nthreads)
        if not h:
            raise ValueError("reference constructor threw std::logic_error")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.qslref_destroy(self.h)
            self.h = None

    @property
    def n(self):
        return self.lib.qslref_num_qubits(self.h)

    def get_state(self) -> np.ndarray:
        out = np.empty(self.lib.qslref_dim(self.h), dtype=self.dtype)
        self.lib.qslref_get_state(self.h, _ptr(out))
        return out

    def set_state(self, st) -> None:
        st = np.ascontiguousarray(st, dtype=self.dtype)
        if self.lib.qslref_set_state(self.h, _ptr(st), st.size) != 0:
            raise ValueError("setState threw std::logic_error")

    def gate(self, name: str, q1: int, q2: int = 0, angle: float = 0.0) -> None:
        rc = self.lib.qslref_gate(self.h, name.encode(), q1, q2 if q2 is not None else 0,
                                  float(angle))
        if rc != 0:
            raise ValueError(f"gate {name} not available on this backend")

    def prob(self, targ, outcome):
        return self.lib.qslref_prob(self.h, targ, outcome)

    def measure(self, targ):
        return self.lib.qslref_measure(self.h, targ)

    def postselect(self, targ, outcome):
        return self.lib.qslref_postselect(self.h, targ, outcome)

    def measure_all(self):
        return int(self.lib.qslref_measure_all(self.h))

    def sample_all(self, nshots) -> dict:
        cap = 1 << max(self.n, 1)
        keys = np.zeros(min(cap, nshots) + 1, dtype=np.uint64)
        cnt = np.zeros_like(keys)
        m = self.lib.qslref_sample_all(self.h, nshots, _ptr(keys), _ptr(cnt), keys.size)
        return {int(k): int(c) for k, c in zip(keys[:m], cnt[:m])}

    def sample_all2(self, nshots) -> dict:
        cap = 1 << self.n
        keys = np.zeros(cap, dtype=np.uint64)
        cnt = np.zeros_like(keys)
        m = self.lib.qslref_sample_all2(self.h, nshots, _ptr(keys), _ptr(cnt), cap)
        return {int(k): int(c) for k, c in zip(keys[:m], cnt[:m])}

    def sample(self, targ, nshots):
        c = np.zeros(2, dtype=np.uint64)
        self.lib.qslref_sample(self.h, targ, nshots, _ptr(c))
        return c

    def reset(self):
        self.lib.qslref_reset(self.h)

    def set_basis(self, idx):
        if self.lib.qslref_set_basis(self.h, idx) != 0:
            raise ValueError("setBasisState threw")

    def num_ones(self):
        return self.lib.qslref_num_ones(self.h)

    def set_num_ones(self, w):
        if self.lib.qslref_set_num_ones(self.h, w) != 0:
            raise ValueError("setNumOnes threw")

    # Resize backend (resize.hpp:160-180, :310, :350)
    def add_qubit(self, t):
        assert self.lib.qslref_add_qubit(self.h, t) == 0

    def append_qubit(self):
        assert self.lib.qslref_append_qubit(self.h) == 0

    def measure_out(self, t):
        return self.lib.qslref_measure_out(self.h, t)

    def postselect_out(self, t, o):
        return self.lib.qslref_postselect_out(self.h, t, o)

    def reallocate(self):
        assert self.lib.qslref_reallocate(self.h) == 0


def ref_lib():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            raise FileNotFoundError("reference library not built (needs the reference sources)")
        lib = C.CDLL(REF_SO)
        vp = C.c_void_p
        def sig(name, res, *args):
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = list(args)
        sig("qslref_seed", None, C.c_uint32)
        sig("qslref_set_uniforms", None, vp, C.c_size_t)
        sig("qslref_uniforms_left", C.c_size_t)
        sig("qslref_create", vp, C.c_int, C.c_int, C.c_uint, C.c_uint, C.c_uint)
        sig("qslref_create_from_state", vp, C.c_int, C.c_int, vp, C.c_size_t, C.c_uint)
        sig("qslref_destroy", None, vp)
        sig("qslref_clone", vp, vp)
        sig("qslref_assign", C.c_int, vp, vp)
        sig("qslref_dim", C.c_size_t, vp)
        sig("qslref_num_qubits", C.c_uint, vp)
        sig("qslref_get_state", None, vp, vp)
        sig("qslref_set_state", C.c_int, vp, vp, C.c_size_t)
        sig("qslref_gate", C.c_int, vp, C.c_char_p, C.c_uint, C.c_uint, C.c_double)
        sig("qslref_prob", C.c_double, vp, C.c_uint, C.c_uint)
        sig("qslref_measure", C.c_int, vp, C.c_uint)
        sig("qslref_postselect", C.c_double, vp, C.c_uint, C.c_uint)
        sig("qslref_measure_all", C.c_uint64, vp)
        sig("qslref_sample_all", C.c_size_t, vp, C.c_size_t, vp, vp, C.c_size_t)
        sig("qslref_sample_all2", C.c_size_t, vp, C.c_size_t, vp, vp, C.c_size_t)
        sig("qslref_sample", None, vp, C.c_uint, C.c_size_t, vp)
        sig("qslref_reset", None, vp)
        sig("qslref_set_basis", C.c_int, vp, C.c_uint64)
        sig("qslref_num_ones", C.c_int, vp)
        sig("qslref_set_num_ones", C.c_int, vp, C.c_uint)
        sig("qslref_add_qubit", C.c_int, vp, C.c_uint)
        sig("qslref_append_qubit", C.c_int, vp)
        sig("qslref_measure_out", C.c_int, vp, C.c_uint)
        sig("qslref_postselect_out", C.c_double, vp, C.c_uint, C.c_uint)
        sig("qslref_reallocate", C.c_int, vp)
        sig("qslref_next", C.c_uint64, C.c_uint64)
        sig("qslref_hamming_weight", C.c_uint, C.c_uint64)
        sig("qslref_choose", C.c_uint, C.c_uint, C.c_uint)
        sig("qslref_generate_lookup", C.c_size_t, C.c_uint, C.c_uint, vp, C.c_size_t)
        sig("qslref_check_state_np", C.c_int, vp, C.c_size_t)
        sig("qslref_check_state_size", C.c_int, C.c_size_t)
        sig("qslref_fubini_study", C.c_double, vp, vp, C.c_size_t)
        sig("qslref_results_write", C.c_int, C.c_char_p, C.c_char_p, C.c_char_p, C.c_size_t,
            C.c_size_t, vp, C.c_size_t, vp)
        _ref = lib
    return _ref


def ref_feed_uniforms(u) -> None:
    """Hand the reference's next getNum() calls these values, in order."""
    arr = np.ascontiguousarray(u, dtype=np.float64)
    ref_lib().qslref_set_uniforms(_ptr(arr), arr.size)
