#!/usr/bin/env python3
"""Benchmark of the GB300 qsl backend: gates/s and HBM GB/s at 30 qubits, FP64.

Workload: the plain Default-backend path on a 30-qubit complex128 state
(16 GiB), a seeded layered random circuit of depth 40: per layer one gate
per qubit from {hadamard, rotateX, rotateY, rotateZ, phase} (angles
U[0, 2pi)) and 15 two-qubit gates (controlNot or controlPhase, random
control/target over all qubits).  One step is one layer (45 gates); the
state carries over from step to step, so K = 40 steps is the whole circuit.
After the timed layers the benchmark measures 8 random qubits and draws a
100,000-shot sampleAll, each timed on its own and reported in `config`.

value        gates/s over the K timed layers, state resident in HBM, timed with
             CUDA events on the state's stream (max over ranks).
roofline     the kernel with the largest share of the timed gate time: its
             algorithmic bytes per launch (2 x 16 B x amplitudes the
             reference's loop changes) over its mean launch time, against the
             measured HBM copy bandwidth (MEASURED_PEAKS.json).
e2e          the same metric through the C ABI from pinned host memory: the
             state uploaded with qslc_set_state, K layers, the 8 measurements
             and the sampleAll outcomes read back, all inside the timed region.
cpu_baseline the oracle (a C restatement of the reference's OpenMP backend)
             on the host cores, on a bounded sample of the same circuit.

`--impl reference` times that CPU implementation alone (the reference
cannot be built on the GPU machine), with every host thread, on the same
config and metric: the same W untimed and K timed layers.

`--gpus N` with no launcher around it starts N ranks itself (one per GPU,
under torch.distributed.run); each rank runs an independent replica.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from qsl_gb300 import workloads  # noqa: E402

N_QUBITS = 30
LAYERS = 40
SEED = 20240601
METRIC = "gates/s & HBM GB/s at 30q FP64"
UNIT = "gates/s"


def layers_of(circ, n):
    per = n + n // 2
    return [circ[i:i + per] for i in range(0, len(circ), per)]


def alg_bytes(gate: str, n: int) -> int:
    """Bytes the reference's loop reads and writes for one gate on n qubits
    (complex128): 2 x 16 B x amplitudes it changes."""
    amps = {
        "hadamard": 1 << n, "rotateX": 1 << n, "rotateY": 1 << n, "rotateZ": 1 << n,
        "pauliX": 1 << n, "pauliY": 1 << n,
        "phase": 1 << (n - 1), "pauliZ": 1 << (n - 1),
        "controlNot": 1 << (n - 1), "controlPhase": 1 << (n - 2), "controlZ": 1 << (n - 2),
    }[gate]
    return 2 * 16 * amps


def kernel_of(gate: str) -> str:
    return {"hadamard": "k_pair1<H>", "rotateX": "k_pair1<RX>", "rotateY": "k_pair1<RY>",
            "rotateZ": "k_pair1<RZ>", "phase": "k_diag1<PHASE>", "controlNot": "k_pair2<SWAP>",
            "controlPhase": "k_diag2<PHASE>"}[gate]


# DRAM bytes per launch over algorithmic bytes of the dense one-qubit
# kernel, from an ncu capture of k_pair1 on a dense 26-qubit state (2.086 GB
# moved for 2.147 GB of algorithmic traffic; the traffic scales with the
# amplitude count).  It is not measured by this program: the JSON line says
# so next to the number, and --traffic replaces it with a capture's figure.
K_PAIR1_TRAFFIC_RATIO = 2.086 / 2.147
# The same for the grouped sweep of two rotations on a dense 26-qubit state:
# 1.074 + 1.012 GB of DRAM traffic for the two gates' 2 x 2.147 GB.
K_GROUP2_TRAFFIC_RATIO = (1.074 + 1.012) / (2 * 2.147)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_sample(circ, n, seconds=20.0, threads=None):
    """Time the oracle's OpenMP restatement of the reference on the host
    cores: the circuit's gates in order on a fresh n-qubit state, until
    `seconds` have passed (at least 2 gates).  Returns (gates/s, gates, threads)."""
    import oracle
    oracle.build(reference=False)
    threads = threads or os.cpu_count() or 1
    sim = oracle.PortQubits(n, nthreads=threads)
    sim.gate("rotateX", 0, None, 0.1)          # first touch of the host state
    done, t0 = 0, time.perf_counter()
    for g in circ:
        sim.gate(*g)
        done += 1
        if done >= 2 and time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    return done / dt, done, threads


def run_fused(args, torch, q, stream):
    """The precision form (fused FP32 blocks, FP64 norms and CDF): the layered
    circuit at depth 60 on a 32-qubit complex64 state, k = 5, against the
    plain FP64 path at the same size; infidelity on a 28-qubit instance."""
    n, depth = args.fused_qubits, 60
    circ = workloads.layered_mixed(n, depth, SEED + 4)
    per = n + n // 2
    warm, timed = circ[:3 * per], circ[3 * per:]
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    by_k = {}
    for kk in (4, 5, "5tc"):
        sim = q.Qubits(n, dtype=np.complex64)
        sim.set_stream(stream.cuda_stream)
        sim.set_fusion(5 if kk == "5tc" else kk)
        sim.set_fusion_tc(kk == "5tc")
        workloads.apply(sim, warm)
        sim.flush()
        torch.cuda.synchronize()
        b0 = sim.fused_blocks()
        e0.record(stream)
        workloads.apply(sim, timed)
        sim.flush()
        e1.record(stream)
        torch.cuda.synchronize()
        by_k[kk] = {"ms": e0.elapsed_time(e1), "blocks": sim.fused_blocks() - b0}
        if kk != "5tc":
            del sim
            torch.cuda.empty_cache()
    k = min(by_k, key=lambda kk: by_k[kk]["ms"])
    fused_ms, blocks = by_k[k]["ms"], by_k[k]["blocks"]
    hbm, hbm_kind = peaks()
    # one fused block is one sweep of the complex64 state: 2 x 8 B per amplitude
    block_bytes = 2 * 8 * (1 << n)
    roof = {"bound": "hbm", "kernel": "k_dense_tc" if k == "5tc" else f"k_dense<{k}>",
            "alg_bytes_per_launch": block_bytes,
            "achieved": blocks * block_bytes / (fused_ms * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
            "peak_source": hbm_kind,
            "note": "the block sweeps' mean rate over the timed blocks (queue flushes included)"}
    roof["frac"] = roof["achieved"] / hbm
    su = workloads.uniforms(args.shots, SEED + 5)
    t0 = time.perf_counter()
    sim.sample_shots(su)
    sample_ms = (time.perf_counter() - t0) * 1e3
    del sim
    torch.cuda.empty_cache()
    # plain FP64 (complex128) at the same size: one layer
    plain = q.Qubits(n)
    plain.set_stream(stream.cuda_stream)
    workloads.apply(plain, circ[:per])
    torch.cuda.synchronize()
    e0.record(stream)
    workloads.apply(plain, circ[per:2 * per])
    e1.record(stream)
    torch.cuda.synchronize()
    plain_gps = per / (e0.elapsed_time(e1) * 1e-3)
    del plain
    # infidelity on a 28-qubit instance against the FP64 path (bit for bit
    # the reference's Default backend, by the parity tests)
    m = args.fused_check_qubits
    c28 = workloads.layered_mixed(m, depth, SEED + 4)
    ref = q.Qubits(m)
    workloads.apply(ref, c28)
    f = q.Qubits(m, dtype=np.complex64)
    f.set_fusion(5 if k == "5tc" else k)
    f.set_fusion_tc(k == "5tc")
    workloads.apply(f, c28)
    a = ref.getState()
    b = f.getState().astype(np.complex128)
    fid = abs(np.vdot(a, b)) ** 2 / (np.vdot(a, a).real * np.vdot(b, b).real)
    maxerr = float(np.abs(a - b).max())
    del ref, f, a, b
    fused_gps = len(timed) / (fused_ms * 1e-3)
    return {"nqubits": n, "dtype": "c64 state, FP32 blocks (tensor cores: 3xTF32 tcgen05), "
                                   "FP64 norms/CDF", "k": k,
            "by_k": {str(kk): {"ms": v["ms"], "blocks": v["blocks"],
                               "equivalent_gates_per_s": len(timed) / (v["ms"] * 1e-3)}
                     for kk, v in by_k.items()},
            "depth": depth, "gates_timed": len(timed), "fused_blocks": blocks,
            "gates_per_block": len(timed) / max(blocks, 1), "ms": fused_ms,
            "equivalent_gates_per_s": fused_gps,
            "plain_fp64_gates_per_s_same_size": plain_gps,
            "speedup_vs_plain_fp64": fused_gps / plain_gps,
            "infidelity": 1 - fid, "infidelity_qubits": m, "max_abs_err": maxerr,
            "sample_shots": args.shots, "sample_ms": sample_ms, "roofline": roof}


def run_np(args, torch, q, stream):
    """Number-preserving backend: 28 qubits, weight 14, 2000 gates from
    {npRotateX, swap, phase, controlPhase}; the OpenMP NP restatement of the
    reference on the host cores beside it."""
    n, w, ngates = 28, 14, 2000
    st = workloads.np_gaussian_state(n, w, SEED + 6)
    circ = workloads.np_mix(n, ngates, SEED + 7)
    sim = q.QubitsNP(state=st)
    sim.set_stream(stream.cuda_stream)
    workloads.apply(sim, circ[:50])
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    workloads.apply(sim, circ)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    touched = 0
    for g, _, _, _ in circ:
        from math import comb
        touched += {"npRotateX": 2 * comb(n - 2, w - 1), "swap": 2 * comb(n - 2, w - 1),
                    "phase": comb(n - 1, w - 1), "controlPhase": comb(n - 2, w - 2)}[g]
    out = {"nqubits": n, "nones": w, "gates": ngates, "ms": ms, "gates_per_s": ngates / (ms * 1e-3),
           "alg_gbs": 32 * touched / (ms * 1e-3) / 1e9, "stored_amplitudes": sim.num_stored()}
    del sim
    if not args.no_cpu:
        import oracle
        oracle.build(reference=False)
        thr = os.cpu_count() or 1
        cpu = oracle.PortNPQubits(n, w, nthreads=thr, state=st)
        t0 = time.perf_counter()
        done = 0
        for g in circ:
            cpu.gate(*g)
            done += 1
            if time.perf_counter() - t0 > args.cpu_seconds / 2:
                break
        out["cpu_baseline"] = {"value": done / (time.perf_counter() - t0), "unit": UNIT, "cores": thr,
                               "kind": "port", "sample": f"first {done} gates, OpenMP NP restatement"}
    return out


BATCH_SHOTS = 1024
SM_COUNT = 152


def fp64_peak_gops():
    """The FP64 pipe's rate: 2 operations per SM per clock (a DFMA probe on
    GB300 measured 2.07), at the measured maximum SM clock."""
    mhz = 2070.0
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        mhz = float(json.load(open(p)).get("sm_max_mhz", mhz))
    return 2 * SM_COUNT * mhz * 1e6 / 1e9


def batch_roofline(ns, ls, tile_log2, amp_bytes, kernel_ms, fp64):
    """Roofline of one batch launch.  HBM: an instance above a shared-memory
    tile writes its |0..0> state, reads and writes it twice per layer (two
    passes) and reads it once for the measurements, (2 + 4 L) x 2^n x amp
    bytes; smaller instances never leave shared memory; every instance's
    2^n |a|^2 terms are written and read back once as doubles for the
    sampling CDF, 16 x 2^n bytes.  Arithmetic: the
    FP64 operations the reference's loops perform (12 n 2^n per layer for
    rotateY and rotateZ on every qubit, 4 n 2^n for the probabilities, 4 x
    2^n for the CDF), against the FP64 pipe's rate -- the kernel puts part of
    them on the integer pipes, so this fraction can pass 1."""
    n = np.asarray(ns, dtype=np.int64)
    L = np.asarray(ls, dtype=np.int64)
    big = n > tile_log2
    hbm_bytes = float(np.sum(np.where(big, (2 + 4 * L) << n, 0)) * amp_bytes + np.sum(16 << n))
    # shared memory: a resident state is read and written by each rotateY
    # sweep, by the fused rotateZ sweep and by the ladder, per layer
    smem_bytes = float(np.sum(np.where(big, 0, (L * (n + 2)) << n)) * 2 * amp_bytes)
    ops = float(np.sum((12 * n * L + 4 * n + 4) << n))
    sec = kernel_ms * 1e-3
    hbm, kind = peaks()
    mhz = fp64_peak_gops() / (2 * SM_COUNT) * 1e3
    smem_peak = 128 * SM_COUNT * mhz * 1e6 / 1e9
    out = {"hbm": {"alg_bytes": hbm_bytes, "achieved": hbm_bytes / sec / 1e9, "peak": hbm,
                   "unit": "GB/s", "peak_source": kind},
           "smem": {"alg_bytes": smem_bytes, "achieved": smem_bytes / sec / 1e9, "peak": smem_peak,
                    "unit": "GB/s", "peak_source": "128 B per SM per clock at the measured maximum SM clock"},
           "instances_in_hbm": int(big.sum())}
    for k in ("hbm", "smem"):
        out[k]["frac"] = out[k]["achieved"] / out[k]["peak"]
    if fp64:
        peak = fp64_peak_gops()
        out["fp64"] = {"reference_ops": ops, "achieved": ops / sec / 1e9, "peak": peak,
                       "unit": "Gop/s", "peak_source": "2 FP64 operations per SM per clock at the "
                                                        "measured maximum SM clock"}
    else:
        peak = 128 * SM_COUNT * mhz * 1e6 / 1e9
        out["fp32"] = {"reference_ops": ops, "achieved": ops / sec / 1e9, "peak": peak,
                       "unit": "Gop/s", "peak_source": "128 FP32 operations per SM per clock at the "
                                                        "measured maximum SM clock"}
    arith = "fp64" if fp64 else "fp32"
    out[arith]["frac"] = out[arith]["achieved"] / peak
    out["bound"] = max(("hbm", "smem", arith), key=lambda k: out[k]["frac"])
    return out


def batch_workload(args):
    """The batch section's instances: n uniform in [10, 20], L uniform in
    [4, 16], angles uniform in [0, 2 pi), 1024 uniforms per instance.
    Returns the generator too, which the plain comparison draws from next."""
    rng = np.random.default_rng(SEED + 8)
    ninst = args.batch_instances
    ns = rng.integers(10, 21, ninst).astype(np.uint32)
    ls = rng.integers(4, 17, ninst).astype(np.uint32)
    gates = ls.astype(np.int64) * (3 * ns.astype(np.int64) - 1)
    angles = rng.uniform(0, 2 * np.pi, int(np.sum(2 * ns.astype(np.int64) * ls)))
    u = workloads.uniforms(ninst * BATCH_SHOTS, SEED + 9)
    return rng, ns, ls, gates, angles, u


def run_batch(args, torch, q):
    """The batching form: 4096 independent ansatz circuits, n uniform in
    [10, 20], L uniform in [4, 16] layers of rotateY/rotateZ on every qubit
    plus a controlNot ladder, per-instance angles; every qubit's
    probabilities and 1024 shots per instance; one persistent launch from a
    CUDA graph, complex64 and complex128.  The plain FP64 path (per-gate
    launches through the C ABI) runs a random subset of the same instances."""
    rng, ns, ls, gates, angles, u = batch_workload(args)
    ninst, nshots = args.batch_instances, BATCH_SHOTS
    total_gates = int(gates.sum())
    out = {"instances": ninst, "shots_per_instance": nshots, "total_gates": total_gates,
           "state_bytes_c128": int(np.sum((1 << ns.astype(np.int64)) * 16))}
    for name, dt in (("c64", np.complex64), ("c128", np.complex128)):
        b = q.Batch(ns, ls, nshots, dtype=dt)
        tuned_ms = b.autotune(angles, u)                   # picks the launch shape
        b.run(angles, u)                                  # warm-up replay
        reps = 2
        t0 = time.perf_counter()
        for _ in range(reps):
            b.run(angles, u)
        dt_s = (time.perf_counter() - t0) / reps
        shape = b.shape()
        out[name] = {"s": dt_s, "gates_per_s": total_gates / dt_s, "kernel_ms": tuned_ms,
                     "shape": shape,
                     "roofline": batch_roofline(ns, ls, shape["tile_log2"], 16 if name == "c128" else 8,
                                                tuned_ms, name == "c128")}
        del b
    # plain FP64 path on a random subset, scaled by gate count
    sub = rng.choice(ninst, args.batch_plain_sample, replace=False)
    at = np.concatenate([[0], np.cumsum(2 * ns.astype(np.int64) * ls)])
    t0 = time.perf_counter()
    g = 0
    for i in sub:
        n, L = int(ns[i]), int(ls[i])
        a = angles[at[i]:at[i + 1]].reshape(L, n, 2)
        sim = q.Qubits(n)
        for l in range(L):
            for qq in range(n):
                sim.rotateY(qq, a[l, qq, 0])
            for qq in range(n):
                sim.rotateZ(qq, a[l, qq, 1])
            for qq in range(n - 1):
                sim.controlNot(qq, qq + 1)
        for qq in range(n):
            sim.prob(qq, 0)
            sim.prob(qq, 1)
        sim.sample_shots(u[i * nshots:(i + 1) * nshots])
        g += int(gates[i])
        del sim
    plain_s = time.perf_counter() - t0
    plain_gps = g / plain_s
    out["plain_fp64_gates_per_s"] = plain_gps
    out["plain_sample_instances"] = int(args.batch_plain_sample)
    out["speedup_c64_vs_plain_fp64"] = out["c64"]["gates_per_s"] / plain_gps
    out["speedup_c128_vs_plain_fp64"] = out["c128"]["gates_per_s"] / plain_gps
    return out


def run_batch_sharded(args, torch, q, rep):
    """The batch section on several ranks: the same instances, split by
    cost (qsl_gb300/batch_shards.py), each rank's share as one batch on its
    GPU.  The job's rate is all instances' gates over the slowest rank's
    time; every probability and shot is gathered back in instance order
    after the timed region, and rank 0 then runs the whole batch alone and
    reports whether the reassembled results are its bits."""
    from qsl_gb300 import batch_shards as bs
    _, ns, ls, gates, angles, u = batch_workload(args)
    ninst, nshots = args.batch_instances, BATCH_SHOTS
    total_gates = int(gates.sum())
    parts = bs.partition_by_cost(bs.instance_costs(ns, ls), rep.world)
    mine = parts[rep.rank]
    sub_n, sub_l, sub_a, sub_u = bs.select(ns, ls, angles, u, nshots, mine)
    loads = [int(bs.instance_costs(ns[p], ls[p]).sum()) for p in parts]
    out = {"instances": ninst, "shots_per_instance": nshots, "total_gates": total_gates,
           "ranks": rep.world, "partition": "longest first by L * 2^n",
           "max_over_mean_load": max(loads) / (sum(loads) / len(loads))}
    empty = ([], np.empty((0, nshots), dtype=np.uint64))
    for name, dt in (("c64", np.complex64), ("c128", np.complex128)):
        b = q.Batch(sub_n, sub_l, nshots, dtype=dt) if mine.size else None
        tuned_ms = b.autotune(sub_a, sub_u) if b else 0.0
        if b:
            b.run(sub_a, sub_u)                           # warm-up replay
        rep.barrier()
        torch.cuda.synchronize()
        reps = 2
        t0 = time.perf_counter()
        for _ in range(reps):
            res = b.run(sub_a, sub_u) if b else empty
        torch.cuda.synchronize()
        slowest = rep.max((time.perf_counter() - t0) / reps)
        got = rep.gather(([np.asarray(x) for x in res[0]], np.asarray(res[1])))
        probs, shots = bs.assemble(ns, nshots, parts, got)
        out[name] = {"s": slowest, "gates_per_s": total_gates / slowest,
                     "kernel_ms_slowest_rank": rep.max(tuned_ms)}
        del b
        if rep.leader:
            # the whole batch on this rank alone, after the timed region: the
            # reassembled results must be its bits, instance for instance
            whole = q.Batch(ns, ls, nshots, dtype=dt)
            p1, s1 = whole.run(angles, u)
            same = (all(np.array_equal(a, c) for a, c in zip(probs, p1))
                    and np.array_equal(np.asarray(shots), np.asarray(s1)))
            out[name]["matches_single_rank_run"] = bool(same)
            del whole
        rep.barrier()
    return out


def workload_config(n, steps, warmup, layers):
    """The `config` object, the same in both arms: the circuit, its size and
    the gates the K timed steps run."""
    ngates = sum(len(layers[(warmup + k) % len(layers)]) for k in range(steps))
    return {"workload": f"plain FP64 {n}-qubit layered random circuit (depth {LAYERS}): per layer "
                        f"{n} one-qubit gates + {n // 2} controlNot/controlPhase; one layer per step, "
                        f"layers {warmup}..{warmup + steps - 1} timed after {warmup} untimed",
            "nqubits": n, "state_bytes": (1 << n) * 16, "gates_timed": ngates,
            "l2": f"state ({(1 << n) * 16 / 2**30:g} GiB) is larger than L2 (129 MB); no flush needed"}


def e2e_pinned(n, local_ranks):
    """Whether every local rank may pin a host copy of its state."""
    try:
        ram = os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_PHYS_PAGES")
    except (ValueError, OSError):
        return local_ranks == 1
    return local_ranks * (1 << n) * 16 <= ram // 2


def launch_windows(layer, grouping=True):
    """The calls of one layer with the gates of the kernel each launches.

    The library holds a one-qubit gate back until the next call: a
    one-qubit gate on another qubit joins it in one sweep (k_group2),
    anything else releases it alone.  Before a two-qubit gate, and at the
    end of the layer, a held gate is released by an explicit flush (call
    None), so each timing window holds one kernel.  Returns (call, gates)
    pairs; gates is None for a call that launches nothing."""
    out, held = [], None
    for g, a, b, x in layer:
        gate = (g, a, b, x)
        if b is None and grouping:
            if held is None:
                out.append((gate, None))
                held = gate
            elif held[1] != a:
                out.append((gate, [held, gate]))
                held = None
            else:
                out.append((gate, [held]))
                held = gate
            continue
        if held is not None:
            out.append((None, [held]))
            held = None
        out.append((gate, [gate]))
    if held is not None:
        out.append((None, [held]))
    return out


def roofline_of(args, name, top, peak, peak_kind):
    """The roofline object of the dominant kernel: its algorithmic bytes per
    launch (the reference's count, 2 x 16 B x amplitudes changed, for every
    gate the launch applies) over its mean CUDA-event launch time, against
    the measured HBM copy bandwidth.  A grouped launch applies two gates in
    one read and one write of the state, so its fraction can pass 1 while
    its DRAM traffic is about half its algorithmic bytes.  `traffic` is DRAM
    bytes per launch: --traffic when a capture of this run's kernel is
    given, else the dense-state ratio of an earlier capture scaled to this
    launch, and labelled as such."""
    per_launch = top["bytes"] / top["launches"]
    achieved = per_launch / (top["ms"] / top["launches"] * 1e-3) / 1e9
    out = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
           "frac": achieved / peak, "peak_source": peak_kind,
           "alg_bytes_per_launch": per_launch, "gates_per_launch": top["gates"] / top["launches"]}
    if args.traffic:
        out["traffic"] = args.traffic
        out["traffic_source"] = "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, given with --traffic"
    elif name.startswith("k_pair1"):
        out["traffic"] = per_launch * K_PAIR1_TRAFFIC_RATIO
        out["traffic_source"] = ("scaled from an earlier ncu capture of k_pair1 on a dense 26-qubit "
                                 "state (DRAM bytes / algorithmic bytes = 0.972); not measured in this run")
    elif name == "k_group2":
        out["traffic"] = per_launch * K_GROUP2_TRAFFIC_RATIO
        out["traffic_source"] = ("scaled from an earlier ncu capture of k_group2 (two rotations) on a dense "
                                 "26-qubit state (DRAM bytes / algorithmic bytes of both gates = 0.486: one "
                                 "read and one write of the state); not measured in this run")
    else:
        out["traffic"] = None
        out["traffic_source"] = "no capture of this kernel given"
    return out


def run_gpu(args):
    import torch
    import qsl_gb300 as q

    from qsl_gb300.replicas import Replicas
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    rep = Replicas("nccl")          # one independent replica per GPU; no data-path collective
    rank, world = rep.rank, rep.world
    n = args.qubits
    circ = workloads.layered_mixed(n, LAYERS, rep.seed(SEED))
    layers = layers_of(circ, n)
    stream = torch.cuda.Stream()
    sim = q.Qubits(n)
    sim.set_stream(stream.cuda_stream)

    grouping = os.environ.get("QSLC_GROUP", "1")[:1] != "0"

    def timed(timing, fn, launched):
        """Run fn; with `timing`, inside a pair of events on the stream,
        recorded with the gates of the kernel it launches (None: none)."""
        if timing is None:
            fn()
            return
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        if launched:
            timing.append((launched, e0, e1))

    def run_layer(li, timing):
        for call, launched in launch_windows(layers[li % len(layers)], grouping):
            if call is None:
                timed(timing, sim.flush, launched)
            else:
                timed(timing, lambda: sim.gate(*call), launched)

    # warm-up layers (the circuit's own first layers)
    for w in range(args.warmup):
        run_layer(w, None)
    sim.synchronize()
    torch.cuda.synchronize()
    rep.barrier()

    clocks = ClockSampler()
    clocks.start()
    timing = []
    launches0 = sim.launches()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t_start.record(stream)
    for k in range(args.steps):
        run_layer(args.warmup + k, timing)
    t_end.record(stream)
    torch.cuda.synchronize()
    launches = sim.launches() - launches0
    clk = clocks.stop()
    rep.barrier()
    local_ms = t_start.elapsed_time(t_end)
    ngates = sum(len(layers[(args.warmup + k) % len(layers)]) for k in range(args.steps))
    total_ms = rep.max(local_ms)                      # the slowest rank
    job_gates_per_s = rep.throughput(ngates, local_ms * 1e-3)

    # per-kernel breakdown from the per-launch events; a grouped launch
    # counts the reference's algorithmic bytes of both of its gates
    per = {}
    for gs, e0, e1 in timing:
        ms = e0.elapsed_time(e1)
        name = "k_group2" if len(gs) == 2 else kernel_of(gs[0][0])
        d = per.setdefault(name, {"launches": 0, "ms": 0.0, "bytes": 0, "gates": 0})
        d["launches"] += 1
        d["ms"] += ms
        d["bytes"] += sum(alg_bytes(g[0], n) for g in gs)
        d["gates"] += len(gs)
    gate_ms = sum(d["ms"] for d in per.values())
    top_name, top = max(per.items(), key=lambda kv: kv[1]["ms"])
    peak, peak_kind = peaks()
    all_gbs = sum(d["bytes"] for d in per.values()) / (gate_ms * 1e-3) / 1e9

    # measurement and sampling on the evolved state
    rng = np.random.default_rng(SEED)
    mq = [int(x) for x in rng.choice(n, 8, replace=False)]
    mu = workloads.uniforms(8, SEED + 1)
    su = workloads.uniforms(args.shots, SEED + 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    outs = [sim.measure(a, float(u)) for a, u in zip(mq, mu)]
    t1 = time.perf_counter()
    shots = sim.sample_shots(su)
    t2 = time.perf_counter()

    # end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        # pinned host memory for every local rank's 16 GiB state only while
        # that stays under half of the host's memory; pageable above that
        pinned = e2e_pinned(n, int(os.environ.get("LOCAL_WORLD_SIZE", world)))
        host = torch.empty((1 << n) * 2, dtype=torch.float64, pin_memory=pinned)
        hv = host.numpy().view(np.complex128)
        hv[:] = 0
        hv[0] = 1
        sim2 = q.Qubits(n)
        sim2.set_stream(stream.cuda_stream)
        # one untimed upload first, as the device leg's warm-up steps: the
        # first copies out of a freshly pinned buffer ran at 44-58 GB/s on
        # a GB300, later ones at about 210 GB/s
        sim2.L.qslc_set_state(sim2.h, hv.ctypes.data, hv.size)
        torch.cuda.synchronize()
        e0 = time.perf_counter()
        sim2.L.qslc_set_state(sim2.h, hv.ctypes.data, hv.size)
        for k in range(args.steps):
            for g, a, b, x in layers[k % len(layers)]:
                sim2.gate(g, a, b, x)
        o2 = [sim2.measure(a, float(u)) for a, u in zip(mq, mu)]
        sh2 = sim2.sample_shots(su)
        e1 = time.perf_counter()
        g2 = sum(len(layers[k % len(layers)]) for k in range(args.steps))
        e2e = {"value": g2 / (e1 - e0), "unit": UNIT,
               "h2d_bytes_per_step": int(hv.nbytes / args.steps),
               "d2h_bytes_per_step": int((sh2.nbytes + 8 * len(o2)) / args.steps),
               "includes": f"qslc_set_state of the {(1 << n) * 16 >> 30} GiB state from "
                           f"{'pinned' if pinned else 'pageable'} host memory, K layers, "
                           "8 measurements, 100k-shot sampleAll read back; one untimed upload "
                           "of the same buffer before"}
        del sim2, host

    line = {
        "metric": METRIC, "value": job_gates_per_s, "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(n, args.steps, args.warmup, layers),
        "parallelism": "replicas" if world > 1 else "single GPU",
        "detail": {
            "hbm_gbs_all_gates": all_gbs,
            "measure8_ms": (t1 - t0) * 1e3, "measure_outcomes": outs,
            "sample_shots": args.shots, "sample_ms": (t2 - t1) * 1e3,
            "kernels": {k: {"launches": v["launches"], "ms": v["ms"],
                            "gbs": v["bytes"] / (v["ms"] * 1e-3) / 1e9,
                            "share": v["ms"] / gate_ms} for k, v in per.items()},
        },
        "roofline": roofline_of(args, top_name, top, peak, peak_kind),
        "gpu_launches": launches,
        "clocks": clk,
    }
    if e2e:
        line["e2e"] = e2e
    del sim
    torch.cuda.empty_cache()
    if not args.no_fused:
        line["fused"] = run_fused(args, torch, q, stream)
    if not args.no_np:
        line["np"] = run_np(args, torch, q, stream)
    if not args.no_batch:
        line["batch"] = (run_batch(args, torch, q) if world == 1
                         else run_batch_sharded(args, torch, q, rep))
    if rank == 0 and not args.no_cpu:
        v, done, thr = cpu_sample(circ, n, seconds=args.cpu_seconds)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": thr, "kind": "port",
                                "sample": f"first {done} gates of the same {n}-qubit circuit, "
                                          f"OpenMP restatement of the reference's Omp backend"}
    rep.close()
    if rep.leader:
        print(json.dumps(line), flush=True)


def run_reference(args):
    """The reference's CPU algorithm on every host thread: the oracle's C
    restatement of the reference's OpenMP backend (the reference's own
    sources are not on the GPU machine).  It runs the GPU arm's workload
    exactly: the same circuit, W untimed layers, then K timed layers of 45
    gates each, on a state that starts at |0...0>.  --ref-gates G > 0 bounds
    a step to the first G gates of its layer instead (the config then says
    so)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    oracle.build(reference=False)
    n = args.qubits
    circ = workloads.layered_mixed(n, LAYERS, SEED)
    layers = layers_of(circ, n)
    threads = os.cpu_count() or 1
    sim = oracle.PortQubits(n, nthreads=threads)
    per_step = args.ref_gates if args.ref_gates > 0 else None

    def step(li):
        gates = layers[li % len(layers)][:per_step]
        for g in gates:
            sim.gate(*g)
        return len(gates)

    for w in range(args.warmup):
        step(w)
    k = 0
    t0 = time.perf_counter()
    for s in range(args.steps):
        k += step(args.warmup + s)
    dt = time.perf_counter() - t0
    v = k / dt
    config = workload_config(n, args.steps, args.warmup, layers)
    if per_step:
        config["workload"] += f"; reference arm: the first {per_step} gates of each layer only"
        config["gates_timed"] = k
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config, "parallelism": f"OpenMP, {threads} host threads",
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{k} gates: {'the first %d gates of ' % per_step if per_step else ''}"
                                   f"layers {args.warmup}..{args.warmup + args.steps - 1}"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def free_port() -> int:
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def launch_ranks(nranks: int, argv, script: str | None = None) -> int:
    """Start `nranks` local ranks of `script` (this file by default) under
    torch.distributed.run, one per GPU (each rank binds LOCAL_RANK), with the
    rendezvous on 127.0.0.1; returns the launcher's exit status."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           f"--nproc-per-node={nranks}", "--master-addr", "127.0.0.1",
           "--master-port", str(free_port()), script or os.path.abspath(__file__), *argv]
    return subprocess.call(cmd)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=LAYERS)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--qubits", type=int, default=N_QUBITS)
    ap.add_argument("--shots", type=int, default=100_000)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-gates", type=int, default=0,
                    help="reference arm: time only the first G gates of each layer (0: whole layers)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fused", action="store_true")
    ap.add_argument("--no-np", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-instances", type=int, default=4096)
    ap.add_argument("--batch-plain-sample", type=int, default=48)
    ap.add_argument("--fused-qubits", type=int, default=32)
    ap.add_argument("--fused-check-qubits", type=int, default=28)
    ap.add_argument("--traffic", type=float, default=None,
                    help="dram bytes per launch of the top kernel from an ncu capture")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # --gpus N without a launcher: start N ranks here, one per GPU
        sys.exit(launch_ranks(args.gpus, sys.argv[1:]))
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
