// qslc_internal.cuh -- shared definitions of the CUDA state-vector backend.
//
// Layout in HBM: one contiguous array of complex amplitudes, {re, im}
// interleaved (qsl::complex<Fp>, include/qsl/utils/complex.hpp:40-49 of
// qsl), 16 B per amplitude for complex128 and 8 B for complex64.  A plain
// state holds all 2^n amplitudes; a number-preserving (NP) state holds only
// the C(n, w) amplitudes of Hamming weight w, in ascending order of their
// basis index (the order of qsl's generateLookup, src/utils/misc.cpp:75-90).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <string>

#include "qslc.h"
#include "fusion_host.hpp"

#include <vector>

namespace qslc {

// ---------------------------------------------------------------------------
// Errors: every entry point returns a status; the message is kept per thread.
// ---------------------------------------------------------------------------
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

#define QSLC_CUDA(call)                                   \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) return qslc::cuda_fail(e_, #call); \
    } while (0)

// ---------------------------------------------------------------------------
// Entry points: every status-returning C function opens an NVTX range named
// after itself (visible in Nsight timelines; a no-op with no tool attached)
// and honours host-side fault injection.  QSLC_FORCE_ERROR=name[:code[:after]]
// makes the entry point `name` (or every one, for "*") return `code`
// (default QSLC_ECUDA) once `after` calls of it have succeeded, with a
// message saying so -- so callers' error paths can be tested without a GPU
// fault.  It is read once, when the library is loaded.
// ---------------------------------------------------------------------------
int forced_error(const char *entry);

struct NvtxRange {
    explicit NvtxRange(const char *name);
    ~NvtxRange();
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

#define QSLC_ENTRY(name)                                              \
    qslc::NvtxRange qslc_nvtx_range_(name);                           \
    if (int qslc_forced_ = qslc::forced_error(name)) return qslc_forced_

// ---------------------------------------------------------------------------
// Round-to-nearest arithmetic with no contraction: qsl's x86-64 build rounds
// every product and every sum on its own, and so must we to produce the
// same bits.
// ---------------------------------------------------------------------------
template <class T> struct rn;
template <> struct rn<double> {
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
};
template <> struct rn<float> {
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
};

template <class T> struct cplx_t;
template <> struct cplx_t<double> { using type = double2; };
template <> struct cplx_t<float> { using type = float2; };
template <class T> using cplx = typename cplx_t<T>::type;

// ---------------------------------------------------------------------------
// Bit insertion: the pair index j in [0, 2^(n-1)) becomes the basis index
// with a 0 at bit t; the reference's nested (s, r) loops (gates.cpp:36-37)
// visit the same indices in the same order.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint64_t insert0(uint64_t j, unsigned t)
{
    uint64_t low = j & ((uint64_t(1) << t) - 1);
    return ((j >> t) << (t + 1)) | low;
}
// two zero bits at lo < hi
__host__ __device__ __forceinline__ uint64_t insert00(uint64_t j, unsigned lo, unsigned hi)
{
    return insert0(insert0(j, lo), hi);
}

// ---------------------------------------------------------------------------
// The state object behind a qslc_state handle.
// ---------------------------------------------------------------------------
struct Scratch {
    void *ptr = nullptr;
    size_t bytes = 0;
    int ensure(size_t need);   // grows with cudaMalloc; QSLC_EOOM on failure
    void release();
};

// Device tables of a number-preserving state (np.cu): the reference's five
// lookup tables {n-1,w-1}, {n-2,w-1}, {n-2,w-2}, {n-1,w}, {n,w}.
struct NPTables {
    unsigned n = 0, w = 0;
    uint32_t *tab[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    uint64_t len[5] = {0, 0, 0, 0, 0};
};

}  // namespace qslc

struct qslc_state {
    unsigned n = 0;           // qubits
    int dtype = QSLC_C128;    // QSLC_C128 or QSLC_C64
    int np = 0;               // 1: number-preserving (compressed) layout
    unsigned nones = 0;       // Hamming weight of an NP state
    uint64_t namps = 0;       // live amplitudes (2^n, or C(n, w) for NP)
    uint64_t cap = 0;         // amplitudes allocated (>= namps)
    int resizable = 0;        // 1: qubits may be added and removed (resize.cu)
    void *amps = nullptr;     // device amplitudes
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int device = 0;
    qslc::Scratch scratch;    // reductions, CDF tiles
    qslc::Scratch scratch2;
    void *host_pinned = nullptr;  // small device->host results
    size_t host_pinned_bytes = 0;
    uint64_t launches = 0;    // kernels launched through this handle
    qslc::NPTables *npt = nullptr;
    // precision form (fused.cu): queued gates, fusion width, block matrices
    unsigned fuse_k = 0;
    int fuse_tc = 1;          // five-qubit blocks on the tensor cores (fused_tc.cu)
    std::vector<qslc::GateOp> fuse_queue;
    qslc::Scratch fuse_mats;
    qslc::Scratch fuse_tc_mats;   // packed tensor-core operands, then an error word
    uint64_t fused_blocks = 0;
    // a one-qubit gate held back to run in one sweep with the next
    // one-qubit gate on another qubit (gates.cu, k_group2)
    qslc::GateOp held{};
    bool has_held = false;
    int *wait_err = nullptr;         // device word set by a staged sweep whose barrier wait ran out
    bool wait_err_pending = false;   // staged sweeps launched since the word was last read

    size_t amp_bytes() const { return dtype == QSLC_C128 ? 16 : 8; }
};

namespace qslc {

// Launch geometry: grid-stride loops over `work` items with 256 threads per
// CTA and at most 16 resident CTAs per SM on the 152-SM part.
unsigned sm_count();
inline unsigned grid_for(uint64_t work, unsigned threads = 256, unsigned per_sm = 16)
{
    uint64_t blocks = (work + threads - 1) / threads;
    uint64_t cap = uint64_t(sm_count()) * per_sm;
    if (blocks > cap) blocks = cap;
    if (blocks == 0) blocks = 1;
    return unsigned(blocks);
}

int ensure_pinned(qslc_state *s, size_t bytes);

// The device word staged sweeps set when a barrier wait runs out (allocated
// on first use, zeroed); wait_error() reads and clears it on the host.
int ensure_wait_err(qslc_state *s);
int wait_error(qslc_state *s);

// gates.cu
int launch_gate1(qslc_state *s, int gate, unsigned targ, double angle);
int launch_gate2(qslc_state *s, int gate, unsigned q1, unsigned q2, double angle);
// two one-qubit gates on different qubits, in this order, in one sweep
int launch_group2(qslc_state *s, const GateOp &g0, const GateOp &g1);
bool grouping_enabled();
// Debug builds (-DQSLC_DEBUG_BOUNDS): QSLC_EINVAL when a sweep met an index
// outside its state since the last call; QSLC_OK otherwise and in default
// builds.
int debug_bounds_error();
int launch_collapse(qslc_state *s, unsigned targ, unsigned outcome, double factor);
// complex64 collapse with the factor applied in double (precision form)
int launch_collapse_f64(qslc_state *s, unsigned targ, unsigned outcome, double factor);
int launch_fill_basis(qslc_state *s, uint64_t pos);

// fused.cu
int fusion_flush(qslc_state *s);

// resize.cu
int resize_add_qubit(qslc_state *s, unsigned targ);
int resize_collapse_out(qslc_state *s, unsigned targ, unsigned outcome, double factor, bool f64);
int resize_reallocate(qslc_state *s);
int resize_capacity(qslc_state *s, uint64_t count);   // grow the allocation; contents undefined

// fused_tc.cu
void tc_pack_block(const std::vector<cd> &U, float *out);
size_t tc_block_floats();
bool tc_usable(const qslc_state *s);
int tc_launch(qslc_state *s, const float *d_b, const unsigned *pos, int *d_err);

// measure.cu
int seq_prob(qslc_state *s, unsigned targ, unsigned outcome, double *out);
int seq_sample_all(qslc_state *s, const double *u_host, uint64_t nshots, uint64_t *out_host);
int seq_sample_all2(qslc_state *s, const double *u_host, uint64_t nshots, uint64_t *out_host);

// np.cu
int np_init_tables();
int np_prepare(qslc_state *s, unsigned w);   // build the tables for weight w
void np_release(qslc_state *s);
int np_gate(qslc_state *s, int gate, unsigned q1, unsigned q2, double angle);
int np_collapse(qslc_state *s, unsigned targ, unsigned outcome, double factor);
int np_prob(qslc_state *s, unsigned targ, unsigned outcome, double *out);
int np_sample_all(qslc_state *s, const double *u, uint64_t n, uint64_t *out);
int np_sample_all2(qslc_state *s, const double *u, uint64_t n, uint64_t *out);
int np_expand(qslc_state *s, void *host_full);
int np_compress(qslc_state *s, const void *host_full, unsigned w);
uint64_t np_choose(unsigned n, unsigned k);
uint64_t np_rank_host(uint64_t x);

}  // namespace qslc
