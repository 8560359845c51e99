/*
 * qslc.h -- C ABI of the GB300 state-vector backend for qsl.
 *
 * The reference library (lanamineh/qsl) exposes its simulators only as the
 * C++ class template qsl::Qubits<Type, Fp>; it has no C or foreign-function
 * interface.  These entry points are the narrowest boundary that carries
 * that member API across a shared-library edge: an opaque handle, plain
 * pointers and sizes, and an int status.  include/qsl/qubits/cuda.hpp
 * rebuilds qsl::Qubits on top of them, and any FFI (ctypes, cgo, JNI) can
 * bind them directly.  Each declaration names the qsl member it stands for
 * (file:line inside the qsl project).
 *
 * Numerics: amplitudes, probabilities and sampled outcomes are the bits the
 * reference's Default backend produces on the same inputs (every product
 * and sum is rounded on its own, Hadamard divides by sqrt(2), sums run in
 * the reference's order), given the same uniforms for measurement.
 *
 * Threading: one handle is one CUDA stream.  Gate calls are asynchronous;
 * calls that return host values synchronise that stream.  A handle must not
 * be used from two threads at once (qsl's objects are not thread-safe
 * either).
 */
#ifndef QSLC_H
#define QSLC_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define QSLC_API __attribute__((visibility("default")))
#else
#define QSLC_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct qslc_state qslc_state;

/* status codes */
enum {
    QSLC_OK = 0,
    QSLC_EINVAL = 1,   /* bad argument: qubit index, size, gate code, weight */
    QSLC_EOOM = 2,     /* device allocation failed */
    QSLC_ECUDA = 3,    /* CUDA runtime error (message in qslc_last_error) */
    QSLC_ETIMEOUT = 4, /* a bounded device-side wait gave up */
    QSLC_ENOTNP = 5,   /* state is not number preserving (quantum.cpp:133-156) */
    QSLC_ESIZE = 6     /* state size mismatch (default.cpp:70-74, :98-102) */
};

/* amplitude types: qsl::complex<double> and qsl::complex<float> */
enum { QSLC_C128 = 0, QSLC_C64 = 1 };

/* gate codes; names follow the qsl::Qubits members */
enum {
    /* one-qubit gates, qslc_gate1 (default.hpp:208-333) */
    QSLC_PAULI_X = 0,
    QSLC_PAULI_Y = 1,
    QSLC_PAULI_Z = 2,
    QSLC_HADAMARD = 3,
    QSLC_PHASE = 4,
    QSLC_ROTATE_X = 5,
    QSLC_ROTATE_Y = 6,
    QSLC_ROTATE_Z = 7,
    /* two-qubit gates, qslc_gate2 (default.hpp:354-608); for the control*
     * gates q1 is the control and q2 the target */
    QSLC_CONTROL_NOT = 16,
    QSLC_CONTROL_Y = 17,
    QSLC_CONTROL_Z = 18,
    QSLC_CONTROL_ROTATE_X = 19,
    QSLC_CONTROL_ROTATE_Y = 20,
    QSLC_CONTROL_ROTATE_Z = 21,
    QSLC_CONTROL_PHASE = 22,
    QSLC_CONTROL_HADAMARD = 23,
    QSLC_SWAP = 24,
    QSLC_FSWAP = 25,
    QSLC_NP_ROTATE_X = 26,
    QSLC_NP_ROTATE_Y = 27,
    QSLC_NP_HADAMARD = 28
};

/* Library version, e.g. 100 for 0.1.0. */
QSLC_API int qslc_version(void);

/* Message of the last failed call on this thread ("" if none). */
QSLC_API const char *qslc_last_error(void);

/* Qubits(unsigned nqubits): the all-zero state |0...0>
 * (default.cpp:39-46).  dtype is QSLC_C128 or QSLC_C64. */
QSLC_API int qslc_create(unsigned nqubits, int dtype, qslc_state **out);

/* NP Qubits(unsigned nqubits, unsigned nones): the basis state with the
 * nones lowest bits set (np.cpp:42-55, :69-79).  EINVAL unless
 * 1 <= nones < nqubits, as the reference throws.  Only the C(n, nones)
 * amplitudes of that weight are stored on the device. */
QSLC_API int qslc_create_np(unsigned nqubits, unsigned nones, int dtype, qslc_state **out);

/* ~Qubits */
QSLC_API int qslc_destroy(qslc_state *s);

/* Qubits(const Qubits&) (default.hpp:137): a deep device-to-device copy. */
QSLC_API int qslc_clone(const qslc_state *src, qslc_state **out);

/* operator=(const Qubits&) (default.cpp:94-105): copies the amplitudes;
 * QSLC_ESIZE when the qubit counts differ (the reference throws). */
QSLC_API int qslc_assign(qslc_state *dst, const qslc_state *src);

/* getNumQubits (default.cpp:114-118) */
QSLC_API unsigned qslc_num_qubits(const qslc_state *s);

/* 1 for a number-preserving state */
QSLC_API int qslc_is_np(const qslc_state *s);

/* QSLC_C128 or QSLC_C64 */
QSLC_API int qslc_dtype(const qslc_state *s);

/* Amplitudes held on the device: 2^n, or C(n, w) for an NP state. */
QSLC_API uint64_t qslc_num_stored(const qslc_state *s);

/* NP getNumOnes / setNumOnes (np.cpp:148-165); setNumOnes re-initialises
 * to the lowest basis state of the new weight. */
QSLC_API int qslc_num_ones(const qslc_state *s, unsigned *out);
QSLC_API int qslc_set_num_ones(qslc_state *s, unsigned nones);

/* reset (default.cpp:57-65; np.cpp:69-79) */
QSLC_API int qslc_reset(qslc_state *s);

/* setState (default.cpp:67-78; np.cpp:81-98).  `amps` points to n_amps
 * host amplitudes of the handle's type; QSLC_ESIZE unless n_amps == 2^n.
 * An NP state takes its new weight from the input, and QSLC_ENOTNP when
 * the nonzero amplitudes have different weights. */
QSLC_API int qslc_set_state(qslc_state *s, const void *amps, uint64_t n_amps);

/* getState (default.cpp:108-112): writes all 2^n amplitudes to `amps`. */
QSLC_API int qslc_get_state(const qslc_state *s, void *amps, uint64_t n_amps);

/* setBasisState (default.cpp:80-90; np.cpp:100-116) */
QSLC_API int qslc_set_basis(qslc_state *s, uint64_t index);

/* One-qubit gate: pauliX, ..., rotateZ (gates.cpp:32-209; np/gates.cpp:33-113).
 * `angle` is ignored by the gates without one.  On a plain state the gate
 * may be held back until the handle's next call: a one-qubit gate on
 * another qubit then runs with it in one sweep, with the same bits as two;
 * any other call applies it first.  qslc_flush or qslc_synchronize apply a
 * held gate without another call; QSLC_GROUP=0 in the environment turns
 * the holding off. */
QSLC_API int qslc_gate1(qslc_state *s, int gate, unsigned targ, double angle);

/* Two-qubit gate (gates.cpp:215-682; np/gates.cpp:118-415).  EINVAL when
 * q1 == q2 or either index is out of range. */
QSLC_API int qslc_gate2(qslc_state *s, int gate, unsigned q1, unsigned q2, double angle);

/* prob(targ, outcome) (measure.cpp:126-147; np/measure.cpp:141-168).  The
 * result is the reference's sequential sum, bit for bit; a complex64 state
 * returns its float value widened to double. */
QSLC_API int qslc_prob(qslc_state *s, unsigned targ, unsigned outcome, double *out);

/* The collapse step of measure/postselect (measure.cpp:31-57;
 * np/measure.cpp:32-70): scale the `outcome` half by `factor`, zero the
 * other half. */
QSLC_API int qslc_collapse(qslc_state *s, unsigned targ, unsigned outcome, double factor);

/* measure(targ) (measure.cpp:81-107) with the uniform `u` that
 * random.getNum() would return (:91). */
QSLC_API int qslc_measure(qslc_state *s, unsigned targ, double u, int *outcome);

/* postselect(targ, outcome) (measure.cpp:149-161); returns the probability. */
QSLC_API int qslc_postselect(qslc_state *s, unsigned targ, unsigned outcome, double *prob);

/* Resizeable states: the qubit-count operations of qsl's Resize backend
 * (include/qsl/qubits/resize.hpp:46-370).  A resizeable handle keeps a
 * capacity of allocated amplitudes, 2^n of them live, and accepts in
 * qslc_set_state any power-of-two size and in qslc_assign another
 * resizeable state of any size (resize.cpp:67-78).  Gates and measurement
 * are the Default backend's (resize/gates.cpp, resize/measure.cpp repeat
 * default/ line for line).  The calls below return QSLC_EINVAL on a handle
 * not made by qslc_create_resizable. */
QSLC_API int qslc_create_resizable(unsigned nqubits, int dtype, qslc_state **out);
QSLC_API int qslc_is_resizable(const qslc_state *s);
/* allocated amplitudes (the reference's dim_max) */
QSLC_API uint64_t qslc_capacity(const qslc_state *s);

/* addQubit(targ) (resize.cpp:106-147): a new qubit in |0> at position
 * targ <= n; the old qubits at and above targ move up by one.  The
 * capacity doubles when it is full.  appendQubit() is targ = n. */
QSLC_API int qslc_add_qubit(qslc_state *s, unsigned targ);

/* collapseOut(targ, outcome, factor) (resize/measure.cpp:61-95): keep the
 * amplitudes with bit targ = outcome, scaled by factor, and remove the
 * qubit.  EINVAL on a one-qubit state. */
QSLC_API int qslc_collapse_out(qslc_state *s, unsigned targ, unsigned outcome, double factor);

/* measureOut(targ) (resize/measure.cpp:156-182) with the uniform `u`. */
QSLC_API int qslc_measure_out(qslc_state *s, unsigned targ, double u, int *outcome);

/* postselectOut(targ, outcome) (resize/measure.cpp:238-251); returns the
 * probability. */
QSLC_API int qslc_postselect_out(qslc_state *s, unsigned targ, unsigned outcome, double *prob);

/* reallocateState (resize.cpp:92-98): shrink the capacity to 2^n. */
QSLC_API int qslc_reallocate(qslc_state *s);

/* sample(targ, nsamples) (measure.cpp:191-216): counts[0], counts[1] for
 * the nshots uniforms u[0..nshots). */
QSLC_API int qslc_sample(qslc_state *s, unsigned targ, const double *u, uint64_t nshots,
                uint64_t counts[2]);

/* sampleAll(nsamples) (measure.cpp:220-234; np/measure.cpp:243-256): the
 * basis index drawn by each uniform, in order, into out[0..nshots).  The
 * reference folds these into a std::map of counts. */
QSLC_API int qslc_sample_all(qslc_state *s, const double *u, uint64_t nshots, uint64_t *out);

/* sampleAll2(nsamples) (measure.cpp:237-267; np/measure.cpp:259-289): the
 * bin each uniform falls in under the reference's merge of sorted uniforms
 * against an Fp running sum -- the first basis index whose running sum
 * exceeds u -- into out[0..nshots), in the order of u.  A uniform at or
 * above the total falls in no bin (the reference counts it nowhere) and
 * reads back as UINT64_MAX.  The reference returns a std::map with every
 * index as a key; count the outcomes to rebuild it. */
QSLC_API int qslc_sample_all2(qslc_state *s, const double *u, uint64_t nshots, uint64_t *out);

/* measureAll (measure.cpp:110-123): draw one index with `u`, then collapse
 * to that basis state. */
QSLC_API int qslc_measure_all(qslc_state *s, double u, uint64_t *outcome);

/* Stream control.  `stream` is a cudaStream_t; NULL selects the handle's
 * own stream. */
QSLC_API int qslc_set_stream(qslc_state *s, void *stream);
QSLC_API void *qslc_get_stream(const qslc_state *s);
QSLC_API int qslc_synchronize(qslc_state *s);

/* Kernels launched through this handle since it was created. */
QSLC_API uint64_t qslc_launch_count(const qslc_state *s);

/* No counterpart in the reference (its getState returns a copy,
 * default.hpp:165): the device address of the stored amplitudes, for
 * zero-copy interop (a framework tensor over the state, a device-side
 * comparison).  There are qslc_num_stored amplitudes of 16 (QSLC_C128) or 8
 * (QSLC_C64) bytes; queued precision-form gates are applied first.  The
 * address changes when a call reallocates the state (setNumOnes, addQubit,
 * reallocate, assignment between sizes); work on it must be ordered after
 * the handle's stream. */
QSLC_API int qslc_device_amps(qslc_state *s, void **out);

/* Precision form (no counterpart in the reference).  With max_qubits in
 * 1..5 on a complex64 plain state, gates are queued and, at the next call
 * that reads or measures the state (or qslc_flush), fused into dense
 * blocks of at most max_qubits qubits applied as one FP32 sweep each;
 * prob, measurement decisions, collapse factors and the sampling CDF run in
 * FP64.  Results then match the FP64 path to FP32 accuracy instead of bit
 * for bit.  0 turns fusion off (after applying what is queued). */
QSLC_API int qslc_set_fusion(qslc_state *s, unsigned max_qubits);
QSLC_API int qslc_flush(qslc_state *s);
/* Five-qubit blocks on states of 12 qubits or more run on the tensor cores
 * (tcgen05, 3xTF32 split with FP32 accumulation); this is the default.
 * on = 0 applies them on the CUDA cores instead. */
QSLC_API int qslc_set_fusion_tc(qslc_state *s, int on);
/* Fused blocks applied through this handle so far. */
QSLC_API uint64_t qslc_fused_blocks(const qslc_state *s);

/* Batching form (no counterpart in the reference).  A batch of `ninst`
 * independent circuits, instance i on nqubits[i] qubits (2..26) with
 * nlayers[i] layers of: rotateY on every qubit, rotateZ on every qubit,
 * controlNot(q, q+1) for q = 0..n-2; then prob(q, 0) and prob(q, 1) for
 * every q and `nshots` sampleAll draws.  All instances run in one
 * persistent kernel, followed by one kernel that walks the sampling CDFs,
 * both captured once in a CUDA graph.  Results are the bits qsl's Default
 * backend gives for the same calls.  Device memory: the instances' inputs
 * and results, 8 bytes per amplitude of every instance (the |a|^2 terms
 * of the CDFs), and two state buffers per CTA of the largest instance
 * when it does not fit a shared-memory tile. */
typedef struct qslc_batch qslc_batch;
QSLC_API int qslc_batch_create(int dtype, uint32_t ninst, const uint32_t *nqubits,
                               const uint32_t *nlayers, uint32_t nshots, qslc_batch **out);
/* angles: per instance, layer-major, per qubit (rotateY angle, rotateZ
 * angle); uniforms: nshots per instance.  probs: per instance 2*n values
 * (prob(q,0), prob(q,1)), q ascending; shots: nshots per instance, in the
 * order of the uniforms.  The call's host work (coefficients, sorting each
 * instance's uniforms, reordering the shots) runs on up to 32 host threads
 * it starts and joins before it returns. */
QSLC_API int qslc_batch_run(qslc_batch *b, const double *angles, const double *uniforms,
                            double *probs, uint64_t *shots);
/* Measure every launch shape (threads per CTA, shared-memory tile of 64 or
 * 128 KB, CTAs per SM) on this batch with these inputs and keep the fastest;
 * best_ms receives its time for one run.  No reference counterpart. */
QSLC_API int qslc_batch_autotune(qslc_batch *b, const double *angles, const double *uniforms,
                                 double *best_ms);
/* Use one launch shape; QSLC_EINVAL unless it is one the autotuner would
 * try for this batch. */
QSLC_API int qslc_batch_set_shape(qslc_batch *b, unsigned threads, unsigned tile_log2,
                                  unsigned ctas_per_sm);
/* The launch shape in use: threads per CTA, log2 of the tile's amplitudes,
 * CTAs per SM and the grid. */
QSLC_API int qslc_batch_shape(const qslc_batch *b, unsigned *threads, unsigned *tile_log2,
                              unsigned *ctas_per_sm, unsigned *grid);
QSLC_API int qslc_batch_destroy(qslc_batch *b);

/* No counterpart in the reference: prob(targ, outcome) for callers that
 * cannot allocate device memory -- code running inside a framework whose
 * pool or arena owns every device allocation, code that must not trigger
 * the device-wide synchronisation cudaMalloc/cudaFree can cause, plugins in
 * a process that has reserved the whole device.  `amps` is the caller's
 * device array of 2^nqubits amplitudes (dtype QSLC_C128 or QSLC_C64),
 * `stream` a cudaStream_t (NULL: the default stream); the result is the
 * same bits as qslc_prob.  It allocates nothing: its scratch is one
 * file-scope device array of QSLC_NOALLOC_SCRATCH_BYTES, which every GPU
 * that loads the library holds until the process exits, shared by all
 * calls (calls that overlap on the GPU race on it; calls made through this
 * library in one process are serialised).  States above
 * QSLC_NOALLOC_MAX_QUBITS qubits (and nqubits == 0) are rejected with
 * QSLC_EINVAL before anything else is done.  Each call blocks until the
 * result is on the host: it synchronises `stream` and copies into fixed
 * host arrays, so it must not be called while that stream (or, in global
 * capture mode, any stream) is being captured.  The first call on a device
 * looks up the array's address on that device and keeps it for the life of
 * the process; do not use the library across a cudaDeviceReset. */
#define QSLC_NOALLOC_SCRATCH_BYTES (1u << 20)
#define QSLC_NOALLOC_MAX_QUBITS 27
QSLC_API int qslc_prob_noalloc(const void *amps, unsigned nqubits, int dtype, unsigned targ,
                               unsigned outcome, void *stream, double *out);

#ifdef __cplusplus
}
#endif
#endif /* QSLC_H */
