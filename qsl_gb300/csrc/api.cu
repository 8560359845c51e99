// api.cu -- the extern "C" entry points declared in include/qslc.h.
//
// Host-side validation happens before any launch: qubit indices, distinct
// qubits for two-qubit gates, sizes and Hamming weights.  The reference
// validates only sizes and weights (it throws std::logic_error,
// src/qubits/default/default.cpp:70-74, np.cpp:48-50); an out-of-range qubit
// index there is undefined behaviour, here it is QSLC_EINVAL.
#include "qslc_internal.cuh"

#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

namespace qslc {

static thread_local std::string g_err;

void set_error(const std::string &msg) { g_err = msg; }

int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *what)
{
    g_err = std::string("CUDA error ") + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) +
            ") in " + what;
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return QSLC_EOOM;
    }
    return QSLC_ECUDA;
}

NvtxRange::NvtxRange(const char *name) { nvtxRangePushA(name); }
NvtxRange::~NvtxRange() { nvtxRangePop(); }

namespace {

struct ForcedError {
    std::string entry;          // entry point name, or "*"
    int code = 0;               // 0: nothing forced
    long long after = 0;        // calls that succeed first
    std::atomic<long long> seen{0};

    ForcedError()
    {
        const char *e = std::getenv("QSLC_FORCE_ERROR");
        if (!e || !*e) return;
        std::string v(e);
        const size_t c1 = v.find(':');
        entry = v.substr(0, c1);
        code = QSLC_ECUDA;
        if (c1 != std::string::npos) {
            const size_t c2 = v.find(':', c1 + 1);
            code = std::atoi(v.substr(c1 + 1, c2 == std::string::npos ? std::string::npos : c2 - c1 - 1).c_str());
            if (c2 != std::string::npos) after = std::atoll(v.c_str() + c2 + 1);
        }
        if (code <= 0) code = QSLC_ECUDA;
    }
};

ForcedError &forced()
{
    static ForcedError f;
    return f;
}

const int forced_init = (forced(), 0);   // read the variable when the library loads

}  // namespace

int forced_error(const char *name)
{
    ForcedError &f = forced();
    if (!f.code || (f.entry != "*" && f.entry != name)) return 0;
    if (f.seen.fetch_add(1) < f.after) return 0;
    g_err = std::string("forced failure of ") + name + " (QSLC_FORCE_ERROR)";
    return f.code;
}

unsigned sm_count()
{
    static unsigned v = [] {
        int d = 0, c = 0;
        cudaGetDevice(&d);
        if (cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, d) != cudaSuccess || c <= 0)
            c = 152;
        return unsigned(c);
    }();
    return v;
}

int Scratch::ensure(size_t need)
{
    if (bytes >= need && ptr) return QSLC_OK;
    release();
    size_t grow = need + need / 4 + 4096;
    if (cudaMalloc(&ptr, grow) != cudaSuccess) {
        cudaGetLastError();
        ptr = nullptr;
        bytes = 0;
        return fail(QSLC_EOOM, "out of device memory for scratch (" + std::to_string(grow) + " bytes)");
    }
    bytes = grow;
    return QSLC_OK;
}

int ensure_wait_err(qslc_state *s)
{
    if (s->wait_err) return QSLC_OK;
    void *p = nullptr;
    if (cudaMalloc(&p, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        return fail(QSLC_EOOM, "out of device memory for the wait error word");
    }
    s->wait_err = static_cast<int *>(p);
    QSLC_CUDA(cudaMemsetAsync(s->wait_err, 0, sizeof(int), s->stream));
    return QSLC_OK;
}

int wait_error(qslc_state *s)
{
    if (!s->wait_err_pending || !s->wait_err) return QSLC_OK;
    s->wait_err_pending = false;
    int h = 0;
    QSLC_CUDA(cudaMemcpyAsync(&h, s->wait_err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    QSLC_CUDA(cudaStreamSynchronize(s->stream));
    if (!h) return QSLC_OK;
    QSLC_CUDA(cudaMemsetAsync(s->wait_err, 0, sizeof(int), s->stream));
    return fail(QSLC_ETIMEOUT, "a staged sweep's shared-memory barrier wait ran out; the state is undefined");
}

void Scratch::release()
{
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

}  // namespace qslc

using namespace qslc;

namespace {

constexpr unsigned MAX_QUBITS = 40;

int check_handle(const qslc_state *s)
{
    if (!s) return fail(QSLC_EINVAL, "null qslc_state handle");
    return QSLC_OK;
}

// Launch the one-qubit gate held back for grouping, alone.
int release_held(qslc_state *s)
{
    if (!s->has_held) return QSLC_OK;
    s->has_held = false;
    return launch_gate1(s, s->held.code, s->held.q1, s->held.angle);
}

// Apply held and queued gates (the gate held for grouping; the precision
// form's queue) before the state is read, and report a staged sweep whose
// barrier wait ran out since the last check.
int flushed(qslc_state *s)
{
    int hrc = release_held(s);
    if (!hrc) hrc = debug_bounds_error();
    if (hrc) return hrc;
    if (!s->fuse_queue.empty()) {
        int rc = fusion_flush(s);
        if (rc) return rc;
    }
    return wait_error(s);
}

// (Re)allocate the amplitude array for `count` amplitudes.
int alloc_amps(qslc_state *s, uint64_t count)
{
    if (count == 0) return fail(QSLC_EINVAL, "no amplitudes to allocate");
    if (s->amps && s->cap == count) {
        s->namps = count;
        return QSLC_OK;
    }
    if (s->amps) cudaFree(s->amps);
    s->amps = nullptr;
    s->namps = 0;
    s->cap = 0;
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, count * s->amp_bytes());
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(QSLC_EOOM, "out of device memory for " + std::to_string(count) + " amplitudes (" +
                                   std::to_string(count * s->amp_bytes()) + " bytes)");
    }
    s->amps = p;
    s->namps = count;
    s->cap = count;
    return QSLC_OK;
}

int new_state(unsigned n, int dtype, qslc_state **out)
{
    if (!out) return fail(QSLC_EINVAL, "null output pointer");
    *out = nullptr;
    if (n < 1 || n > MAX_QUBITS)
        return fail(QSLC_EINVAL, "number of qubits must be in [1, " + std::to_string(MAX_QUBITS) + "]");
    if (dtype != QSLC_C128 && dtype != QSLC_C64) return fail(QSLC_EINVAL, "unknown dtype");
    auto *s = new (std::nothrow) qslc_state();
    if (!s) return fail(QSLC_EOOM, "host allocation failed");
    s->n = n;
    s->dtype = dtype;
    cudaGetDevice(&s->device);
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete s;
        return cuda_fail(e, "cudaStreamCreateWithFlags");
    }
    s->own_stream = true;
    *out = s;
    return QSLC_OK;
}

void free_state(qslc_state *s)
{
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    np_release(s);
    if (s->wait_err) cudaFree(s->wait_err);
    if (s->amps) cudaFree(s->amps);
    s->scratch.release();
    s->scratch2.release();
    s->fuse_mats.release();
    s->fuse_tc_mats.release();
    if (s->host_pinned) cudaFreeHost(s->host_pinned);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

// Weight of the nonzero amplitudes of a full host vector (quantum.cpp:133-156):
// -1 when two nonzero amplitudes differ in weight, -2 when all are zero.
template <class T>
int host_weight(const void *amps, uint64_t dim)
{
    const T *a = static_cast<const T *>(amps);
    int w = -2;
    for (uint64_t i = 0; i < dim; i++) {
        volatile T re2 = a[2 * i] * a[2 * i];
        volatile T im2 = a[2 * i + 1] * a[2 * i + 1];
        T p = re2 + im2;
        if (p != 0) {
            int hw = __builtin_popcountll(i);
            if (w == -2) w = hw;
            else if (w != hw) return -1;
        }
    }
    return w;
}

int np_set_weight(qslc_state *s, unsigned w)
{
    if (w < 1 || w >= s->n)
        return fail(QSLC_EINVAL, "The number of ones must be 1 <= nones < nqubits.");
    int rc = alloc_amps(s, np_choose(s->n, w));
    if (rc) return rc;
    rc = np_prepare(s, w);
    if (rc) return rc;
    s->nones = w;
    return QSLC_OK;
}

int check_q(const qslc_state *s, unsigned q)
{
    if (q >= s->n)
        return fail(QSLC_EINVAL, "qubit index " + std::to_string(q) + " out of range for " +
                                     std::to_string(s->n) + " qubits");
    return QSLC_OK;
}

bool is_np_gate(int g)
{
    switch (g) {
    case QSLC_PAULI_Z: case QSLC_ROTATE_Z: case QSLC_PHASE: case QSLC_CONTROL_Z:
    case QSLC_CONTROL_ROTATE_Z: case QSLC_CONTROL_PHASE: case QSLC_SWAP: case QSLC_FSWAP:
    case QSLC_NP_ROTATE_X: case QSLC_NP_ROTATE_Y: case QSLC_NP_HADAMARD:
        return true;
    default:
        return false;
    }
}

// measure.cpp:81-107, the decision and the factor in Fp
template <class T>
void decide(double p0d, double ud, int *outcome, double *factor)
{
    const T p0 = T(p0d), u = T(ud);
    if (u < p0) {
        *outcome = 0;
        *factor = double(T(1) / std::sqrt(p0));
    } else {
        *outcome = 1;
        *factor = double(T(1) / std::sqrt(T(1) - p0));
    }
}

}  // namespace

extern "C" {

int qslc_version(void) { return 100; }

const char *qslc_last_error(void) { return g_err.c_str(); }

int qslc_create(unsigned nqubits, int dtype, qslc_state **out)
{
    QSLC_ENTRY("qslc_create");
    int rc = new_state(nqubits, dtype, out);
    if (rc) return rc;
    qslc_state *s = *out;
    rc = alloc_amps(s, uint64_t(1) << nqubits);
    if (!rc) rc = launch_fill_basis(s, 0);
    if (rc) {
        free_state(s);
        *out = nullptr;
    }
    return rc;
}

int qslc_create_np(unsigned nqubits, unsigned nones, int dtype, qslc_state **out)
{
    QSLC_ENTRY("qslc_create_np");
    if (nqubits > 32)
        return fail(QSLC_EINVAL, "number-preserving states support at most 32 qubits");
    if (nones < 1 || nones >= nqubits)
        return fail(QSLC_EINVAL, "The number of ones must be 1 <= nones < nqubits.");
    int rc = new_state(nqubits, dtype, out);
    if (rc) return rc;
    qslc_state *s = *out;
    s->np = 1;
    rc = np_set_weight(s, nones);
    if (!rc) rc = launch_fill_basis(s, 0);   // rank of (1 << nones) - 1 is 0
    if (rc) {
        free_state(s);
        *out = nullptr;
    }
    return rc;
}

int qslc_destroy(qslc_state *s)
{
    free_state(s);
    return QSLC_OK;
}

int qslc_clone(const qslc_state *src, qslc_state **out)
{
    QSLC_ENTRY("qslc_clone");
    int rc = check_handle(src);
    if (!rc) rc = flushed(const_cast<qslc_state *>(src));
    if (rc) return rc;
    rc = new_state(src->n, src->dtype, out);
    if (rc) return rc;
    qslc_state *s = *out;
    s->np = src->np;
    s->resizable = src->resizable;
    if (src->np) rc = np_set_weight(s, src->nones);
    else rc = alloc_amps(s, src->namps);
    if (!rc) {
        s->fuse_k = src->fuse_k;
        s->fuse_tc = src->fuse_tc;
    }
    if (!rc) {
        cudaStreamSynchronize(src->stream);
        cudaError_t e = cudaMemcpyAsync(s->amps, src->amps, src->namps * src->amp_bytes(),
                                        cudaMemcpyDeviceToDevice, s->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "clone copy");
    }
    if (rc) {
        free_state(s);
        *out = nullptr;
    }
    return rc;
}

int qslc_assign(qslc_state *dst, const qslc_state *src)
{
    QSLC_ENTRY("qslc_assign");
    int rc = check_handle(dst);
    if (!rc) rc = check_handle(src);
    if (rc) return rc;
    if (dst->dtype != src->dtype || dst->np != src->np || dst->resizable != src->resizable)
        return fail(QSLC_EINVAL, "cannot assign between different simulator types");
    // a resizeable state takes the other's qubit count (resize.hpp: the
    // implicit assignment copies nqubits and dim)
    if (dst->n != src->n && !dst->resizable)
        return fail(QSLC_ESIZE, "Cannot assign Qubits object vector from different number of qubits");
    if (dst == src) return flushed(dst);
    rc = flushed(const_cast<qslc_state *>(src));
    if (rc) return rc;
    dst->fuse_queue.clear();                 // overwritten below
    dst->has_held = false;
    if (dst->resizable && dst->namps != src->namps) {
        rc = resize_capacity(dst, src->namps);
        if (rc) return rc;
        dst->n = src->n;
        dst->namps = src->namps;
    }
    if (dst->np && dst->nones != src->nones) {
        rc = np_set_weight(dst, src->nones);
        if (rc) return rc;
    }
    QSLC_CUDA(cudaStreamSynchronize(src->stream));
    QSLC_CUDA(cudaMemcpyAsync(dst->amps, src->amps, src->namps * src->amp_bytes(),
                              cudaMemcpyDeviceToDevice, dst->stream));
    return QSLC_OK;
}

unsigned qslc_num_qubits(const qslc_state *s) { return s ? s->n : 0; }
int qslc_is_np(const qslc_state *s) { return s ? s->np : 0; }
int qslc_dtype(const qslc_state *s) { return s ? s->dtype : -1; }
uint64_t qslc_num_stored(const qslc_state *s) { return s ? s->namps : 0; }

int qslc_num_ones(const qslc_state *s, unsigned *out)
{
    QSLC_ENTRY("qslc_num_ones");
    int rc = check_handle(s);
    if (rc) return rc;
    if (!s->np) return fail(QSLC_EINVAL, "not a number-preserving state");
    *out = s->nones;
    return QSLC_OK;
}

int qslc_set_num_ones(qslc_state *s, unsigned nones)
{
    QSLC_ENTRY("qslc_set_num_ones");
    int rc = check_handle(s);
    if (rc) return rc;
    if (!s->np) return fail(QSLC_EINVAL, "not a number-preserving state");
    rc = np_set_weight(s, nones);
    if (rc) return rc;
    return launch_fill_basis(s, 0);
}

int qslc_reset(qslc_state *s)
{
    QSLC_ENTRY("qslc_reset");
    int rc = check_handle(s);
    if (rc) return rc;
    s->fuse_queue.clear();
    s->has_held = false;
    return launch_fill_basis(s, 0);
}

int qslc_set_state(qslc_state *s, const void *amps, uint64_t n_amps)
{
    QSLC_ENTRY("qslc_set_state");
    int rc = check_handle(s);
    if (rc) return rc;
    uint64_t dim = uint64_t(1) << s->n;
    if (!amps) return fail(QSLC_EINVAL, "null amplitude pointer");
    if (n_amps != dim && s->resizable) {
        // any power of two (resize.cpp:67-78, quantum.cpp:109-130)
        if (n_amps < 2 || (n_amps & (n_amps - 1)) || n_amps > (uint64_t(1) << MAX_QUBITS))
            return fail(QSLC_ESIZE, "State vector size is not a power of two");
        rc = resize_capacity(s, n_amps);
        if (rc) return rc;
        s->n = unsigned(__builtin_ctzll(n_amps));
        s->namps = dim = n_amps;
    }
    if (n_amps != dim)
        return fail(QSLC_ESIZE, "Cannot assign state vector from different number of qubits");
    s->fuse_queue.clear();
    s->has_held = false;
    if (!s->np) {
        QSLC_CUDA(cudaMemcpyAsync(s->amps, amps, dim * s->amp_bytes(), cudaMemcpyHostToDevice, s->stream));
        QSLC_CUDA(cudaStreamSynchronize(s->stream));
        return QSLC_OK;
    }
    int w = s->dtype == QSLC_C128 ? host_weight<double>(amps, dim) : host_weight<float>(amps, dim);
    if (w == -1) return fail(QSLC_ENOTNP, "Input state is not number preserving.");
    if (w < 0) return fail(QSLC_EINVAL, "state has no nonzero amplitude");
    if (unsigned(w) != s->nones) {
        rc = np_set_weight(s, unsigned(w));
        if (rc) return rc;
    }
    return np_compress(s, amps, unsigned(w));
}

int qslc_get_state(const qslc_state *cs, void *amps, uint64_t n_amps)
{
    QSLC_ENTRY("qslc_get_state");
    int rc = check_handle(cs);
    if (rc) return rc;
    qslc_state *s = const_cast<qslc_state *>(cs);
    const uint64_t dim = uint64_t(1) << s->n;
    if (n_amps != dim) return fail(QSLC_ESIZE, "output size must be 2^nqubits amplitudes");
    if (!amps) return fail(QSLC_EINVAL, "null amplitude pointer");
    rc = flushed(s);
    if (rc) return rc;
    if (s->np) return np_expand(s, amps);
    QSLC_CUDA(cudaMemcpyAsync(amps, s->amps, dim * s->amp_bytes(), cudaMemcpyDeviceToHost, s->stream));
    QSLC_CUDA(cudaStreamSynchronize(s->stream));
    return QSLC_OK;
}

int qslc_set_basis(qslc_state *s, uint64_t index)
{
    QSLC_ENTRY("qslc_set_basis");
    int rc = check_handle(s);
    if (rc) return rc;
    if (s->n < 64 && index >= (uint64_t(1) << s->n))
        return fail(QSLC_EINVAL, "basis index out of range");
    s->fuse_queue.clear();
    s->has_held = false;
    if (!s->np) return launch_fill_basis(s, index);
    const unsigned w = unsigned(__builtin_popcountll(index));
    if (w != s->nones) {
        rc = np_set_weight(s, w);
        if (rc) return rc;
    }
    return launch_fill_basis(s, np_rank_host(index));
}

int qslc_gate1(qslc_state *s, int gate, unsigned targ, double angle)
{
    QSLC_ENTRY("qslc_gate1");
    int rc = check_handle(s);
    if (!rc) rc = check_q(s, targ);
    if (rc) return rc;
    if (gate < QSLC_PAULI_X || gate > QSLC_ROTATE_Z)
        return fail(QSLC_EINVAL, "not a one-qubit gate code: " + std::to_string(gate));
    if (s->np) {
        if (!is_np_gate(gate))
            return fail(QSLC_EINVAL, "gate " + std::to_string(gate) +
                                         " does not preserve the number of ones");
        return np_gate(s, gate, targ, targ, angle);
    }
    if (s->fuse_k) {
        s->fuse_queue.push_back(GateOp{gate, targ, targ, angle});
        return QSLC_OK;
    }
    if (!grouping_enabled()) return launch_gate1(s, gate, targ, angle);
    // one-qubit gates on different qubits run two to a sweep: hold this
    // one until the next call, which either joins it or releases it
    const GateOp g{gate, targ, targ, angle};
    if (s->has_held) {
        s->has_held = false;
        if (s->held.q1 != targ) return launch_group2(s, s->held, g);
        rc = launch_gate1(s, s->held.code, s->held.q1, s->held.angle);
        if (rc) return rc;
    }
    s->held = g;
    s->has_held = true;
    return QSLC_OK;
}

int qslc_gate2(qslc_state *s, int gate, unsigned q1, unsigned q2, double angle)
{
    QSLC_ENTRY("qslc_gate2");
    int rc = check_handle(s);
    if (!rc) rc = check_q(s, q1);
    if (!rc) rc = check_q(s, q2);
    if (rc) return rc;
    if (q1 == q2) return fail(QSLC_EINVAL, "two-qubit gate on a single qubit");
    if (gate < QSLC_CONTROL_NOT || gate > QSLC_NP_HADAMARD)
        return fail(QSLC_EINVAL, "not a two-qubit gate code: " + std::to_string(gate));
    if (s->np) {
        if (!is_np_gate(gate))
            return fail(QSLC_EINVAL, "gate " + std::to_string(gate) +
                                         " does not preserve the number of ones");
        return np_gate(s, gate, q1, q2, angle);
    }
    if (s->fuse_k) {
        s->fuse_queue.push_back(GateOp{gate, q1, q2, angle});
        return QSLC_OK;
    }
    rc = release_held(s);
    if (rc) return rc;
    return launch_gate2(s, gate, q1, q2, angle);
}

int qslc_prob(qslc_state *s, unsigned targ, unsigned outcome, double *out)
{
    QSLC_ENTRY("qslc_prob");
    int rc = check_handle(s);
    if (!rc) rc = check_q(s, targ);
    if (rc) return rc;
    if (outcome > 1) return fail(QSLC_EINVAL, "outcome must be 0 or 1");
    if (!out) return fail(QSLC_EINVAL, "null output pointer");
    rc = flushed(s);
    if (rc) return rc;
    return s->np ? np_prob(s, targ, outcome, out) : seq_prob(s, targ, outcome, out);
}

int qslc_collapse(qslc_state *s, unsigned targ, unsigned outcome, double factor)
{
    QSLC_ENTRY("qslc_collapse");
    int rc = check_handle(s);
    if (!rc) rc = check_q(s, targ);
    if (rc) return rc;
    if (outcome > 1) return fail(QSLC_EINVAL, "outcome must be 0 or 1");
    rc = flushed(s);
    if (rc) return rc;
    if (s->np) return np_collapse(s, targ, outcome, factor);
    if (s->fuse_k && s->dtype == QSLC_C64) return launch_collapse_f64(s, targ, outcome, factor);
    return launch_collapse(s, targ, outcome, factor);
}

int qslc_measure(qslc_state *s, unsigned targ, double u, int *outcome)
{
    QSLC_ENTRY("qslc_measure");
    double p0;
    int rc = qslc_prob(s, targ, 0, &p0);
    if (rc) return rc;
    int o;
    double factor;
    if (s->dtype == QSLC_C128 || s->fuse_k) decide<double>(p0, u, &o, &factor);   // FP64 in the precision form
    else decide<float>(p0, u, &o, &factor);
    rc = qslc_collapse(s, targ, unsigned(o), factor);
    if (rc) return rc;
    if (outcome) *outcome = o;
    return QSLC_OK;
}

int qslc_postselect(qslc_state *s, unsigned targ, unsigned outcome, double *prob)
{
    QSLC_ENTRY("qslc_postselect");
    double p;
    int rc = qslc_prob(s, targ, outcome, &p);
    if (rc) return rc;
    double factor;
    if (s->dtype == QSLC_C128 || s->fuse_k) factor = 1 / std::sqrt(p);   // measure.cpp:154-155
    else factor = double(1.0f / std::sqrt(float(p)));
    rc = qslc_collapse(s, targ, outcome, factor);
    if (rc) return rc;
    if (prob) *prob = p;
    return QSLC_OK;
}

// ---- resizeable states (qsl's Resize backend) ------------------------------

int qslc_create_resizable(unsigned nqubits, int dtype, qslc_state **out)
{
    QSLC_ENTRY("qslc_create_resizable");
    int rc = qslc_create(nqubits, dtype, out);
    if (!rc) (*out)->resizable = 1;
    return rc;
}

int qslc_is_resizable(const qslc_state *s) { return s ? s->resizable : 0; }
uint64_t qslc_capacity(const qslc_state *s) { return s ? s->cap : 0; }

static int check_resizable(const qslc_state *s)
{
    int rc = check_handle(s);
    if (rc) return rc;
    if (!s->resizable) return fail(QSLC_EINVAL, "not a resizeable state");
    return QSLC_OK;
}

int qslc_add_qubit(qslc_state *s, unsigned targ)
{
    QSLC_ENTRY("qslc_add_qubit");
    int rc = check_resizable(s);
    if (rc) return rc;
    if (targ > s->n)
        return fail(QSLC_EINVAL, "new qubit position " + std::to_string(targ) + " above the " +
                                     std::to_string(s->n) + " existing qubits");
    if (s->n + 1 > MAX_QUBITS)
        return fail(QSLC_EINVAL, "at most " + std::to_string(MAX_QUBITS) + " qubits");
    rc = flushed(s);
    if (rc) return rc;
    return resize_add_qubit(s, targ);
}

int qslc_collapse_out(qslc_state *s, unsigned targ, unsigned outcome, double factor)
{
    QSLC_ENTRY("qslc_collapse_out");
    int rc = check_resizable(s);
    if (!rc) rc = check_q(s, targ);
    if (rc) return rc;
    if (outcome > 1) return fail(QSLC_EINVAL, "outcome must be 0 or 1");
    if (s->n < 2) return fail(QSLC_EINVAL, "cannot remove the last qubit");
    rc = flushed(s);
    if (rc) return rc;
    return resize_collapse_out(s, targ, outcome, factor, s->fuse_k && s->dtype == QSLC_C64);
}

int qslc_measure_out(qslc_state *s, unsigned targ, double u, int *outcome)
{
    QSLC_ENTRY("qslc_measure_out");
    int rc = check_resizable(s);
    if (rc) return rc;
    if (s->n < 2) return fail(QSLC_EINVAL, "cannot remove the last qubit");
    double p0;
    rc = qslc_prob(s, targ, 0, &p0);
    if (rc) return rc;
    int o;
    double factor;
    if (s->dtype == QSLC_C128 || s->fuse_k) decide<double>(p0, u, &o, &factor);
    else decide<float>(p0, u, &o, &factor);
    rc = qslc_collapse_out(s, targ, unsigned(o), factor);
    if (rc) return rc;
    if (outcome) *outcome = o;
    return QSLC_OK;
}

int qslc_postselect_out(qslc_state *s, unsigned targ, unsigned outcome, double *prob)
{
    QSLC_ENTRY("qslc_postselect_out");
    int rc = check_resizable(s);
    if (rc) return rc;
    if (s->n < 2) return fail(QSLC_EINVAL, "cannot remove the last qubit");
    double p;
    rc = qslc_prob(s, targ, outcome, &p);
    if (rc) return rc;
    double factor;
    if (s->dtype == QSLC_C128 || s->fuse_k) factor = 1 / std::sqrt(p);   // resize/measure.cpp:243-244
    else factor = double(1.0f / std::sqrt(float(p)));
    rc = qslc_collapse_out(s, targ, outcome, factor);
    if (rc) return rc;
    if (prob) *prob = p;
    return QSLC_OK;
}

int qslc_reallocate(qslc_state *s)
{
    QSLC_ENTRY("qslc_reallocate");
    int rc = check_resizable(s);
    if (!rc) rc = flushed(s);
    if (rc) return rc;
    return resize_reallocate(s);
}

int qslc_sample(qslc_state *s, unsigned targ, const double *u, uint64_t nshots, uint64_t counts[2])
{
    QSLC_ENTRY("qslc_sample");
    if (!counts || (!u && nshots)) return fail(QSLC_EINVAL, "null pointer");
    double p0;
    int rc = qslc_prob(s, targ, 0, &p0);
    if (rc) return rc;
    counts[0] = counts[1] = 0;
    for (uint64_t i = 0; i < nshots; i++) {   // measure.cpp:205-213, compared in Fp
        bool zero = (s->dtype == QSLC_C128 || s->fuse_k) ? (u[i] < p0) : (float(u[i]) < float(p0));
        counts[zero ? 0 : 1]++;
    }
    return QSLC_OK;
}

int qslc_sample_all(qslc_state *s, const double *u, uint64_t nshots, uint64_t *out)
{
    QSLC_ENTRY("qslc_sample_all");
    int rc = check_handle(s);
    if (rc) return rc;
    if (nshots == 0) return QSLC_OK;
    if (!u || !out) return fail(QSLC_EINVAL, "null pointer");
    if (nshots > 0xFFFFFFFFull) return fail(QSLC_EINVAL, "at most 2^32-1 shots per call");
    rc = flushed(s);
    if (rc) return rc;
    if (s->dtype == QSLC_C64 && !s->fuse_k) {
        // the reference draws Fp uniforms; widen the float values exactly
        std::vector<double> uf(nshots);
        for (uint64_t i = 0; i < nshots; i++) uf[i] = double(float(u[i]));
        return s->np ? np_sample_all(s, uf.data(), nshots, out) : seq_sample_all(s, uf.data(), nshots, out);
    }
    return s->np ? np_sample_all(s, u, nshots, out) : seq_sample_all(s, u, nshots, out);
}

int qslc_sample_all2(qslc_state *s, const double *u, uint64_t nshots, uint64_t *out)
{
    QSLC_ENTRY("qslc_sample_all2");
    int rc = check_handle(s);
    if (rc) return rc;
    if (nshots == 0) return QSLC_OK;
    if (!u || !out) return fail(QSLC_EINVAL, "null pointer");
    if (nshots > 0xFFFFFFFFull) return fail(QSLC_EINVAL, "at most 2^32-1 shots per call");
    rc = flushed(s);
    if (rc) return rc;
    std::vector<double> uf;
    const double *uu = u;
    if (s->dtype == QSLC_C64) {     // Fp uniforms, as the reference draws them (:243)
        uf.resize(nshots);
        for (uint64_t i = 0; i < nshots; i++) uf[i] = double(float(u[i]));
        uu = uf.data();
    }
    return s->np ? np_sample_all2(s, uu, nshots, out) : seq_sample_all2(s, uu, nshots, out);
}

int qslc_measure_all(qslc_state *s, double u, uint64_t *outcome)
{
    QSLC_ENTRY("qslc_measure_all");
    uint64_t o = 0;
    int rc = qslc_sample_all(s, &u, 1, &o);
    if (rc) return rc;
    rc = qslc_set_basis(s, o);     // measure.cpp:120
    if (rc) return rc;
    if (outcome) *outcome = o;
    return QSLC_OK;
}

int qslc_set_stream(qslc_state *s, void *stream)
{
    QSLC_ENTRY("qslc_set_stream");
    int rc = check_handle(s);
    if (!rc) rc = flushed(s);
    if (rc) return rc;
    QSLC_CUDA(cudaStreamSynchronize(s->stream));
    if (stream == nullptr) {
        if (!s->own_stream) {
            QSLC_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
            s->own_stream = true;
        }
        return QSLC_OK;
    }
    if (s->own_stream) cudaStreamDestroy(s->stream);
    s->stream = static_cast<cudaStream_t>(stream);
    s->own_stream = false;
    return QSLC_OK;
}

void *qslc_get_stream(const qslc_state *s) { return s ? static_cast<void *>(s->stream) : nullptr; }

int qslc_synchronize(qslc_state *s)
{
    QSLC_ENTRY("qslc_synchronize");
    int rc = check_handle(s);
    if (!rc) rc = flushed(s);
    if (rc) return rc;
    QSLC_CUDA(cudaStreamSynchronize(s->stream));
    return QSLC_OK;
}

uint64_t qslc_launch_count(const qslc_state *s) { return s ? s->launches : 0; }

int qslc_device_amps(qslc_state *s, void **out)
{
    QSLC_ENTRY("qslc_device_amps");
    int rc = check_handle(s);
    if (rc) return rc;
    if (!out) return fail(QSLC_EINVAL, "null output pointer");
    rc = flushed(s);
    if (rc) return rc;
    *out = s->amps;
    return QSLC_OK;
}

int qslc_set_fusion(qslc_state *s, unsigned max_qubits)
{
    QSLC_ENTRY("qslc_set_fusion");
    int rc = check_handle(s);
    if (rc) return rc;
    if (max_qubits > 5) return fail(QSLC_EINVAL, "fusion blocks span at most 5 qubits");
    if (max_qubits && (s->dtype != QSLC_C64 || s->np))
        return fail(QSLC_EINVAL, "the fused precision form runs on complex64 plain states");
    rc = flushed(s);
    if (rc) return rc;
    s->fuse_k = max_qubits;
    return QSLC_OK;
}

int qslc_set_fusion_tc(qslc_state *s, int on)
{
    QSLC_ENTRY("qslc_set_fusion_tc");
    int rc = check_handle(s);
    if (!rc) rc = flushed(s);
    if (rc) return rc;
    s->fuse_tc = on ? 1 : 0;
    return QSLC_OK;
}

int qslc_flush(qslc_state *s)
{
    QSLC_ENTRY("qslc_flush");
    int rc = check_handle(s);
    if (rc) return rc;
    return flushed(s);
}

uint64_t qslc_fused_blocks(const qslc_state *s) { return s ? s->fused_blocks : 0; }

}  // extern "C"
