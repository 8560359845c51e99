// noalloc.cu -- prob() for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: code that runs while its framework
// owns every device allocation (a memory pool or arena that forbids raw
// allocations and would fragment or deadlock on one), code that must not
// synchronize the device the way cudaMalloc/cudaFree can, and plugins
// whose host process has already reserved the whole device.  For them,
// qslc_prob_noalloc runs the same bit-exact sequential-sum machinery as
// qslc_prob on amplitudes the caller owns, with all of its scratch in one
// file-scope device array of fixed size (QSLC_NOALLOC_SCRATCH_BYTES) and
// fixed host arrays.  It allocates nothing: no cudaMalloc, cudaFree, pinned
// host memory or heap.
//
// Rules that follow from the shared, fixed scratch:
//   * the array exists once per device that loads the library and stays
//     allocated until the process exits;
//   * every call reuses it and it keeps the last call's contents; every
//     byte a call reads was written earlier in the same call, so nothing
//     needs clearing between calls;
//   * calls that overlap on the GPU race on it -- a lock serialises calls
//     made through this library in one process, and each call waits for
//     its result before returning, but the scratch must not be shared with
//     anything else;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current, once per device, and
//     keeps it for the life of the process: a cudaDeviceReset (or any other
//     end of the device's primary context) invalidates it, so the library
//     must not be used across a device reset;
//   * every call waits for its result on the host (it synchronises its
//     stream and copies small results into fixed host arrays), so no call
//     may be made while its stream -- or, in global capture mode, any
//     stream -- is being captured into a CUDA graph.
#include <mutex>

#include "seqsum.cuh"

namespace qslc {
namespace {

constexpr uint64_t NOALLOC_MAX_TERMS = uint64_t(1) << 26;   // 2^(n-1) terms: n <= 27
constexpr uint64_t NOALLOC_MAX_TILES = NOALLOC_MAX_TERMS / SEQ_TILE;
constexpr int NOALLOC_FETCH_CAP = 8;

// The device scratch (tile sums, step counts, flags, staged tiles): 1 MiB.
static __device__ __align__(256) unsigned char g_noalloc_scratch[QSLC_NOALLOC_SCRATCH_BYTES];

// Host working storage of the walk, sized for the largest accepted state.
double h_est[NOALLOC_MAX_TILES];
uint64_t h_steps[2 * NOALLOC_MAX_TILES];
uint8_t h_flags[NOALLOC_MAX_TILES];
int16_t h_guess[NOALLOC_MAX_TILES];
uint8_t h_pred[NOALLOC_MAX_TILES];
uint64_t h_slot_tile[NOALLOC_FETCH_CAP];
uint64_t h_batch[NOALLOC_FETCH_CAP];
double h_terms[size_t(NOALLOC_FETCH_CAP) * SEQ_TILE];   // also holds float terms

constexpr int MAX_DEVICES = 64;
void *g_scratch_addr[MAX_DEVICES] = {};
std::mutex g_noalloc_mu;

template <class T>
int prob_noalloc_t(void *scratch, const void *amps, unsigned n, unsigned targ, unsigned outcome,
                   cudaStream_t stream, double *out)
{
    const uint64_t count = uint64_t(1) << (n - 1);
    const uint64_t ntiles = (count + SEQ_TILE - 1) / SEQ_TILE;
    SeqScratch dev = SeqScratch::carve(scratch, ntiles, sizeof(T), NOALLOC_FETCH_CAP);
    if (dev.bytes > QSLC_NOALLOC_SCRATCH_BYTES)
        return fail(QSLC_EINVAL, "state too large for the fixed scratch of qslc_prob_noalloc");
    uint64_t launches = 0;
    SeqEnv<T> env{stream, &launches, dev,
                  SeqHost<T>{h_est, h_steps, h_flags, h_guess, h_pred, h_slot_tile, h_batch,
                             reinterpret_cast<T *>(h_terms), NOALLOC_FETCH_CAP},
                  NOALLOC_FETCH_CAP};
    ProdHalf<T> pr{static_cast<const cplx<T> *>(amps), targ, uint64_t(outcome) << targ};
    T total = T(0);
    auto no_partials = [](uint64_t, T, const T *, uint64_t) {};
    int rc = seq_core<ProdHalf<T>, T, T>(env, pr, count, &total, nullptr, no_partials, nullptr);
    if (rc) return rc;
    *out = double(total);
    return QSLC_OK;
}

}  // namespace
}  // namespace qslc

using namespace qslc;

extern "C" int qslc_prob_noalloc(const void *amps, unsigned nqubits, int dtype, unsigned targ,
                                 unsigned outcome, void *stream, double *out)
{
    if (!amps || !out) return fail(QSLC_EINVAL, "null pointer");
    if (dtype != QSLC_C128 && dtype != QSLC_C64) return fail(QSLC_EINVAL, "unknown dtype");
    if (outcome > 1) return fail(QSLC_EINVAL, "outcome must be 0 or 1");
    // the qubit count is bounded before it is used in any shift
    if (nqubits < 1 || nqubits > QSLC_NOALLOC_MAX_QUBITS)
        return fail(QSLC_EINVAL, "qslc_prob_noalloc accepts 1 to " +
                                     std::to_string(QSLC_NOALLOC_MAX_QUBITS) +
                                     " qubits (its fixed scratch is " +
                                     std::to_string(QSLC_NOALLOC_SCRATCH_BYTES) + " bytes)");
    if (targ >= nqubits) return fail(QSLC_EINVAL, "qubit index out of range");
    static_assert((uint64_t(1) << (QSLC_NOALLOC_MAX_QUBITS - 1)) <= NOALLOC_MAX_TERMS,
                  "the host arrays hold the largest accepted state");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    int dev = 0;
    QSLC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= MAX_DEVICES) return fail(QSLC_EINVAL, "device index out of range");
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        QSLC_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_scratch_addr[dev] = p;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return dtype == QSLC_C128
               ? prob_noalloc_t<double>(g_scratch_addr[dev], amps, nqubits, targ, outcome, st, out)
               : prob_noalloc_t<float>(g_scratch_addr[dev], amps, nqubits, targ, outcome, st, out);
}
