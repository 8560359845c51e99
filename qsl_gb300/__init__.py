"""qsl_gb300 -- a GB300 (sm_103a) state-vector backend for qsl.

The product is the shared library ``libqslc.so`` built from ``csrc/`` and
its C ABI (``include/qslc.h``); C++ users get ``qsl::Qubits<qsl::Type::Cuda,
Fp>`` from ``include/qsl/qubits/cuda.hpp``.  This module binds the same C
ABI with ctypes and mirrors the reference's member API (``pauliX``,
``rotateX``, ``controlNot``, ``prob``, ``measure``, ``sampleAll``, ...) for
Python callers, tests and the benchmark.

There is no CPU fallback: if ``libqslc.so`` is missing, or CUDA reports no
device, constructing a state raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libqslc.so")

C128, C64 = 0, 1
OK, EINVAL, EOOM, ECUDA, ETIMEOUT, ENOTNP, ESIZE = range(7)

GATE1 = {"pauliX": 0, "pauliY": 1, "pauliZ": 2, "hadamard": 3, "phase": 4,
         "rotateX": 5, "rotateY": 6, "rotateZ": 7}
GATE2 = {"controlNot": 16, "controlY": 17, "controlZ": 18, "controlRotateX": 19,
         "controlRotateY": 20, "controlRotateZ": 21, "controlPhase": 22,
         "controlHadamard": 23, "swap": 24, "fswap": 25, "npRotateX": 26,
         "npRotateY": 27, "npHadamard": 28}
ANGLED = {"phase", "rotateX", "rotateY", "rotateZ", "controlRotateX", "controlRotateY",
          "controlRotateZ", "controlPhase", "npRotateX", "npRotateY"}
NP_GATES = ("pauliZ", "rotateZ", "phase", "controlZ", "controlRotateZ", "controlPhase",
            "swap", "fswap", "npRotateX", "npRotateY", "npHadamard")

# every symbol include/qslc.h declares, with its ctypes signature
_VP = C.c_void_p
SIGNATURES = {
    "qslc_version": (C.c_int, []),
    "qslc_last_error": (C.c_char_p, []),
    "qslc_create": (C.c_int, [C.c_uint, C.c_int, C.POINTER(C.c_void_p)]),
    "qslc_create_np": (C.c_int, [C.c_uint, C.c_uint, C.c_int, C.POINTER(C.c_void_p)]),
    "qslc_destroy": (C.c_int, [_VP]),
    "qslc_clone": (C.c_int, [_VP, C.POINTER(C.c_void_p)]),
    "qslc_assign": (C.c_int, [_VP, _VP]),
    "qslc_num_qubits": (C.c_uint, [_VP]),
    "qslc_is_np": (C.c_int, [_VP]),
    "qslc_dtype": (C.c_int, [_VP]),
    "qslc_num_stored": (C.c_uint64, [_VP]),
    "qslc_num_ones": (C.c_int, [_VP, C.POINTER(C.c_uint)]),
    "qslc_set_num_ones": (C.c_int, [_VP, C.c_uint]),
    "qslc_reset": (C.c_int, [_VP]),
    "qslc_set_state": (C.c_int, [_VP, _VP, C.c_uint64]),
    "qslc_get_state": (C.c_int, [_VP, _VP, C.c_uint64]),
    "qslc_set_basis": (C.c_int, [_VP, C.c_uint64]),
    "qslc_gate1": (C.c_int, [_VP, C.c_int, C.c_uint, C.c_double]),
    "qslc_gate2": (C.c_int, [_VP, C.c_int, C.c_uint, C.c_uint, C.c_double]),
    "qslc_prob": (C.c_int, [_VP, C.c_uint, C.c_uint, C.POINTER(C.c_double)]),
    "qslc_collapse": (C.c_int, [_VP, C.c_uint, C.c_uint, C.c_double]),
    "qslc_measure": (C.c_int, [_VP, C.c_uint, C.c_double, C.POINTER(C.c_int)]),
    "qslc_postselect": (C.c_int, [_VP, C.c_uint, C.c_uint, C.POINTER(C.c_double)]),
    "qslc_sample": (C.c_int, [_VP, C.c_uint, _VP, C.c_uint64, _VP]),
    "qslc_sample_all": (C.c_int, [_VP, _VP, C.c_uint64, _VP]),
    "qslc_measure_all": (C.c_int, [_VP, C.c_double, C.POINTER(C.c_uint64)]),
    "qslc_sample_all2": (C.c_int, [_VP, _VP, C.c_uint64, _VP]),
    "qslc_set_stream": (C.c_int, [_VP, _VP]),
    "qslc_get_stream": (C.c_void_p, [_VP]),
    "qslc_synchronize": (C.c_int, [_VP]),
    "qslc_launch_count": (C.c_uint64, [_VP]),
    "qslc_device_amps": (C.c_int, [_VP, C.POINTER(C.c_void_p)]),
    "qslc_prob_noalloc": (C.c_int, [_VP, C.c_uint, C.c_int, C.c_uint, C.c_uint, _VP,
                                    C.POINTER(C.c_double)]),
    "qslc_set_fusion": (C.c_int, [_VP, C.c_uint]),
    "qslc_flush": (C.c_int, [_VP]),
    "qslc_set_fusion_tc": (C.c_int, [_VP, C.c_int]),
    "qslc_fused_blocks": (C.c_uint64, [_VP]),
    "qslc_create_resizable": (C.c_int, [C.c_uint, C.c_int, C.POINTER(C.c_void_p)]),
    "qslc_is_resizable": (C.c_int, [_VP]),
    "qslc_capacity": (C.c_uint64, [_VP]),
    "qslc_add_qubit": (C.c_int, [_VP, C.c_uint]),
    "qslc_collapse_out": (C.c_int, [_VP, C.c_uint, C.c_uint, C.c_double]),
    "qslc_measure_out": (C.c_int, [_VP, C.c_uint, C.c_double, C.POINTER(C.c_int)]),
    "qslc_postselect_out": (C.c_int, [_VP, C.c_uint, C.c_uint, C.POINTER(C.c_double)]),
    "qslc_reallocate": (C.c_int, [_VP]),
    "qslc_batch_create": (C.c_int, [C.c_int, C.c_uint32, _VP, _VP, C.c_uint32,
                                    C.POINTER(C.c_void_p)]),
    "qslc_batch_run": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "qslc_batch_destroy": (C.c_int, [_VP]),
    "qslc_batch_autotune": (C.c_int, [_VP, _VP, _VP, C.POINTER(C.c_double)]),
    "qslc_batch_set_shape": (C.c_int, [_VP, C.c_uint, C.c_uint, C.c_uint]),
    "qslc_batch_shape": (C.c_int, [_VP, C.POINTER(C.c_uint), C.POINTER(C.c_uint),
                                   C.POINTER(C.c_uint), C.POINTER(C.c_uint)]),
}


class QslcError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"qslc error {code}: {msg}")
        self.code = code


class LogicError(QslcError, ValueError):
    """Raised where the reference throws std::logic_error."""


_lib = None


def lib(path: str | None = None):
    """Load libqslc.so (building it first if it is absent and nvcc is present)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        from . import build as _b
        _b.build()
    L = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _check(rc: int) -> None:
    if rc != OK:
        msg = lib().qslc_last_error().decode(errors="replace")
        if rc in (ESIZE, ENOTNP, EINVAL):
            raise LogicError(rc, msg)
        raise QslcError(rc, msg)


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class Qubits:
    """qsl::Qubits on the GPU: the Default-backend member API over the C ABI.

    ``dtype`` is ``np.complex128`` (qsl::complex<double>) or ``np.complex64``
    (qsl::complex<float>).  Methods that draw random numbers in the
    reference (``measure``, ``measureAll``, ``sample``, ``sampleAll``) take
    the uniforms explicitly, or draw them from ``self.rng``.
    """

    _np = False

    def __init__(self, nqubits=None, dtype=np.complex128, state=None, seed=None, _handle=None):
        self.L = lib()
        self.dtype = np.dtype(dtype)
        self.code = C128 if self.dtype == np.complex128 else C64
        self.rng = np.random.default_rng(seed)
        if _handle is not None:
            self.h = _handle
            return
        if state is not None:
            state = np.ascontiguousarray(state, dtype=self.dtype)
            n = state.size.bit_length() - 1
            if state.size != 1 << n:
                raise LogicError(ESIZE, "State vector size is not a power of two")
            nqubits = n
        h = C.c_void_p()
        _check(self._create(nqubits, h))
        self.h = h
        if state is not None:
            self.setState(state)

    def _create(self, n, h):
        return self.L.qslc_create(n, self.code, C.byref(h))

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.L.qslc_destroy(h)
            self.h = None

    def copy(self) -> "Qubits":
        """Qubits(const Qubits&): a deep copy on the device."""
        h = C.c_void_p()
        _check(self.L.qslc_clone(self.h, C.byref(h)))
        q = object.__new__(type(self))
        Qubits.__init__(q, dtype=self.dtype, _handle=h)
        q.rng = np.random.default_rng()
        return q

    def assign(self, other: "Qubits") -> None:
        """operator=(const Qubits&)."""
        _check(self.L.qslc_assign(self.h, other.h))

    # -- state -------------------------------------------------------------
    def getNumQubits(self) -> int:
        return int(self.L.qslc_num_qubits(self.h))

    @property
    def nqubits(self) -> int:
        return self.getNumQubits()

    def reset(self) -> None:
        _check(self.L.qslc_reset(self.h))

    def getState(self) -> np.ndarray:
        out = np.empty(1 << self.nqubits, dtype=self.dtype)
        _check(self.L.qslc_get_state(self.h, _ptr(out), out.size))
        return out

    def setState(self, state) -> None:
        st = np.ascontiguousarray(state, dtype=self.dtype)
        _check(self.L.qslc_set_state(self.h, _ptr(st), st.size))

    def setBasisState(self, index: int) -> None:
        _check(self.L.qslc_set_basis(self.h, index))

    def print(self) -> None:
        print(f"Number of qubits = {self.nqubits}")
        for a in self.getState():
            print(f"{a.real} {a.imag}")

    # -- gates -------------------------------------------------------------
    def gate(self, name: str, q1: int, q2: int | None = None, angle: float = 0.0) -> None:
        if name in GATE1:
            _check(self.L.qslc_gate1(self.h, GATE1[name], q1, float(angle)))
        elif name in GATE2:
            _check(self.L.qslc_gate2(self.h, GATE2[name], q1, q2, float(angle)))
        else:
            raise LogicError(EINVAL, f"unknown gate {name}")

    def synchronize(self) -> None:
        _check(self.L.qslc_synchronize(self.h))

    def launches(self) -> int:
        return int(self.L.qslc_launch_count(self.h))

    def device_amps(self) -> int:
        """Device address of the stored amplitudes (qslc_device_amps)."""
        p = C.c_void_p()
        _check(self.L.qslc_device_amps(self.h, C.byref(p)))
        return int(p.value or 0)

    def num_stored(self) -> int:
        return int(self.L.qslc_num_stored(self.h))

    def device_view(self):
        """A torch tensor over the stored amplitudes, without a copy: shape
        (num_stored, 2), float64 or float32 {re, im} pairs.  Valid while the
        state is not reallocated; order work on it after ``synchronize()``."""
        import torch

        class _CAI:
            pass
        real = "<f8" if self.code == C128 else "<f4"
        holder = _CAI()
        holder.__cuda_array_interface__ = {
            "shape": (self.num_stored(), 2), "typestr": real,
            "data": (self.device_amps(), False), "version": 3, "strides": None}
        t = torch.as_tensor(holder, device="cuda")
        t._qsl_owner = self          # keeps the state alive while the view is
        return t

    def set_stream(self, stream_ptr: int | None) -> None:
        _check(self.L.qslc_set_stream(self.h, stream_ptr))

    def set_fusion(self, max_qubits: int) -> None:
        """Precision form: queue gates and apply them as fused FP32 blocks of
        at most ``max_qubits`` qubits (complex64 states; 0 turns it off)."""
        _check(self.L.qslc_set_fusion(self.h, max_qubits))

    def flush(self) -> None:
        _check(self.L.qslc_flush(self.h))

    def set_fusion_tc(self, on: bool) -> None:
        """Five-qubit fused blocks on the tensor cores (tcgen05; the default)
        or, with False, on the CUDA cores."""
        _check(self.L.qslc_set_fusion_tc(self.h, int(on)))

    def fused_blocks(self) -> int:
        return int(self.L.qslc_fused_blocks(self.h))

    # -- measurement -------------------------------------------------------
    def prob(self, targ: int, outcome: int) -> float:
        out = C.c_double()
        _check(self.L.qslc_prob(self.h, targ, outcome, C.byref(out)))
        return out.value

    def postselect(self, targ: int, outcome: int) -> float:
        out = C.c_double()
        _check(self.L.qslc_postselect(self.h, targ, outcome, C.byref(out)))
        return out.value

    def measure(self, targ: int, u: float | None = None) -> int:
        if u is None:
            u = self.rng.random()
        out = C.c_int()
        _check(self.L.qslc_measure(self.h, targ, float(u), C.byref(out)))
        return out.value

    def measureAll(self, u: float | None = None) -> int:
        if u is None:
            u = self.rng.random()
        out = C.c_uint64()
        _check(self.L.qslc_measure_all(self.h, float(u), C.byref(out)))
        return int(out.value)

    def sample_shots(self, uniforms) -> np.ndarray:
        """The basis index each uniform draws (the shots behind sampleAll)."""
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        out = np.empty(u.size, dtype=np.uint64)
        _check(self.L.qslc_sample_all(self.h, _ptr(u), u.size, _ptr(out)))
        return out

    def sampleAll(self, nsamples: int, uniforms=None) -> dict:
        u = self.rng.random(nsamples) if uniforms is None else uniforms
        shots = self.sample_shots(u)
        keys, counts = np.unique(shots, return_counts=True)
        return {int(k): int(c) for k, c in zip(keys, counts)}

    def sample_shots2(self, uniforms) -> np.ndarray:
        """Bins under sampleAll2's rule; 2**64-1 for a uniform counted nowhere."""
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        out = np.empty(u.size, dtype=np.uint64)
        _check(self.L.qslc_sample_all2(self.h, _ptr(u), u.size, _ptr(out)))
        return out

    def sampleAll2(self, nsamples: int, uniforms=None) -> dict:
        """sampleAll2: counts for every basis index (zeros included), as qsl returns."""
        u = self.rng.random(nsamples) if uniforms is None else uniforms
        shots = self.sample_shots2(u)
        shots = shots[shots != np.uint64(2**64 - 1)]
        keys = self._basis_keys()
        counts = dict.fromkeys((int(k) for k in keys), 0)
        k, c = np.unique(shots, return_counts=True)
        for a, b in zip(k, c):
            counts[int(a)] = int(b)
        return counts

    def _basis_keys(self):
        return np.arange(1 << self.nqubits, dtype=np.uint64)

    def sample(self, targ: int, nsamples: int, uniforms=None) -> list:
        u = np.ascontiguousarray(self.rng.random(nsamples) if uniforms is None else uniforms,
                                 dtype=np.float64)
        counts = np.zeros(2, dtype=np.uint64)
        _check(self.L.qslc_sample(self.h, targ, _ptr(u), u.size, _ptr(counts)))
        return [int(counts[0]), int(counts[1])]


def _mk(name):
    if name in GATE1:
        if name in ANGLED:
            def f(self, targ, angle):
                _check(self.L.qslc_gate1(self.h, GATE1[name], targ, float(angle)))
        else:
            def f(self, targ):
                _check(self.L.qslc_gate1(self.h, GATE1[name], targ, 0.0))
    else:
        if name in ANGLED:
            def f(self, q1, q2, angle):
                _check(self.L.qslc_gate2(self.h, GATE2[name], q1, q2, float(angle)))
        else:
            def f(self, q1, q2):
                _check(self.L.qslc_gate2(self.h, GATE2[name], q1, q2, 0.0))
    f.__name__ = name
    return f


for _g in list(GATE1) + list(GATE2):
    setattr(Qubits, _g, _mk(_g))


class QubitsResize(Qubits):
    """qsl::Qubits<Type::Resize>: the Default arithmetic on a state whose
    qubit count changes (include/qsl/qubits/resize.hpp:46-370).
    ``setState`` takes any power-of-two size, ``assign`` any resizeable
    state."""

    def __init__(self, nqubits=None, dtype=np.complex128, state=None, seed=None, _handle=None):
        if state is not None and nqubits is None:
            st = np.ascontiguousarray(state, dtype=dtype)
            nqubits = max(st.size.bit_length() - 1, 1)
        super().__init__(nqubits, dtype=dtype, state=state, seed=seed, _handle=_handle)

    def _create(self, n, h):
        return self.L.qslc_create_resizable(n, self.code, C.byref(h))

    def capacity(self) -> int:
        """allocated amplitudes (the reference's dim_max)"""
        return int(self.L.qslc_capacity(self.h))

    def addQubit(self, targ: int) -> None:
        _check(self.L.qslc_add_qubit(self.h, targ))

    def appendQubit(self) -> None:
        self.addQubit(self.nqubits)

    def reallocateState(self) -> None:
        _check(self.L.qslc_reallocate(self.h))

    def collapseOut(self, targ: int, outcome: int, factor: float) -> None:
        _check(self.L.qslc_collapse_out(self.h, targ, outcome, float(factor)))

    def measureOut(self, targ: int, u: float | None = None) -> int:
        if u is None:
            u = self.rng.random()
        out = C.c_int()
        _check(self.L.qslc_measure_out(self.h, targ, float(u), C.byref(out)))
        return out.value

    def postselectOut(self, targ: int, outcome: int) -> float:
        out = C.c_double()
        _check(self.L.qslc_postselect_out(self.h, targ, outcome, C.byref(out)))
        return out.value


class QubitsNP(Qubits):
    """qsl::Qubits<Type::NP>: a fixed Hamming weight, stored compressed."""

    _np = True

    def __init__(self, nqubits=None, nones=1, dtype=np.complex128, state=None, seed=None,
                 _handle=None):
        self._nones = nones
        super().__init__(nqubits, dtype=dtype, state=state, seed=seed, _handle=_handle)

    def _create(self, n, h):
        return self.L.qslc_create_np(n, self._nones, self.code, C.byref(h))

    def getNumOnes(self) -> int:
        out = C.c_uint()
        _check(self.L.qslc_num_ones(self.h, C.byref(out)))
        return out.value

    def setNumOnes(self, nones: int) -> None:
        _check(self.L.qslc_set_num_ones(self.h, nones))

    def num_stored(self) -> int:
        return int(self.L.qslc_num_stored(self.h))

    def _basis_keys(self):
        from .workloads import weight_indices
        return weight_indices(self.nqubits, self.getNumOnes()).astype(np.uint64)


class Batch:
    """Batching form: many ansatz circuits (rotateY and rotateZ on every qubit,
    then a controlNot ladder, per layer) in one persistent launch replayed
    from a CUDA graph; per instance prob(q, 0/1) for every q and shots."""

    def __init__(self, nqubits, nlayers, nshots: int, dtype=np.complex128):
        self.L = lib()
        self.n = np.ascontiguousarray(nqubits, dtype=np.uint32)
        self.layers = np.ascontiguousarray(nlayers, dtype=np.uint32)
        self.nshots = int(nshots)
        self.code = C128 if np.dtype(dtype) == np.complex128 else C64
        h = C.c_void_p()
        _check(self.L.qslc_batch_create(self.code, self.n.size, _ptr(self.n), _ptr(self.layers),
                                        self.nshots, C.byref(h)))
        self.h = h
        self.angle_count = int(np.sum(2 * self.n.astype(np.int64) * self.layers))

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.L.qslc_batch_destroy(h)
            self.h = None

    def run(self, angles, uniforms):
        """Returns (probs as a list of (n, 2) arrays, shots as (ninst, nshots))."""
        a = np.ascontiguousarray(angles, dtype=np.float64)
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        assert a.size == self.angle_count and u.size == self.n.size * self.nshots
        probs = np.empty(int(2 * self.n.astype(np.int64).sum()), dtype=np.float64)
        shots = np.empty(self.n.size * self.nshots, dtype=np.uint64)
        _check(self.L.qslc_batch_run(self.h, _ptr(a), _ptr(u), _ptr(probs), _ptr(shots)))
        out, at = [], 0
        for n in self.n:
            out.append(probs[at:at + 2 * n].reshape(n, 2))
            at += 2 * n
        return out, shots.reshape(self.n.size, self.nshots)

    def autotune(self, angles, uniforms) -> float:
        """Time every launch shape on these inputs, keep the fastest; returns
        its milliseconds per run."""
        a = np.ascontiguousarray(angles, dtype=np.float64)
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        ms = C.c_double()
        _check(self.L.qslc_batch_autotune(self.h, _ptr(a), _ptr(u), C.byref(ms)))
        return ms.value

    def set_shape(self, threads: int, tile_log2: int, ctas_per_sm: int) -> None:
        _check(self.L.qslc_batch_set_shape(self.h, threads, tile_log2, ctas_per_sm))

    def shape(self) -> dict:
        v = [C.c_uint() for _ in range(4)]
        _check(self.L.qslc_batch_shape(self.h, *(C.byref(x) for x in v)))
        return dict(zip(("threads", "tile_log2", "ctas_per_sm", "grid"), (x.value for x in v)))

    def shapes(self) -> list:
        """The launch shapes the autotuner tries for this batch."""
        k = 13 if self.code == C128 else 14
        out = []
        for th in (512, 1024):
            for tl, c in ((k - 1, 2), (k - 1, 1), (k, 1)):
                if th * c > 1024 or int(self.n.max()) > 2 * tl:
                    continue
                out.append((th, tl, c))
        return out
