// resize.cu -- changes of the qubit count of a resizeable state, the
// operations of qsl's Resize backend:
//   addQubit      src/qubits/resize/resize.cpp:106-147
//   reallocate    src/qubits/resize/resize.cpp:92-98
//   collapseOut   src/qubits/resize/measure.cpp:61-95
//
// A resizeable state keeps `cap` amplitudes allocated and 2^n of them live,
// like the reference's dim / dim_max pair.  Neither move can run in place in
// parallel (every destination of addQubit lies at or above its source and
// every destination of collapseOut at or below it, so some thread's write
// lands on another thread's unread source), so each kernel reads one
// buffer and writes another: a fresh allocation when the capacity changes,
// else a staging copy of the live amplitudes in the handle's scratch.
#include "qslc_internal.cuh"

namespace qslc {

namespace {

// addQubit(t): old amplitude j moves to j with a 0 inserted at bit t; the
// partner with bit t set becomes 0 (resize.cpp:127-140).
template <class T>
__global__ void __launch_bounds__(256) k_expand(const cplx<T> *__restrict__ src,
                                                cplx<T> *__restrict__ dst, uint64_t nsrc, unsigned t)
{
    const uint64_t bit = uint64_t(1) << t;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    cplx<T> z;
    z.x = T(0);
    z.y = T(0);
    for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < nsrc; j += stride) {
        const uint64_t i = insert0(j, t);
        dst[i] = src[j];
        dst[i | bit] = z;
    }
}

// collapseOut(t, o, f): new amplitude j is old (j with bit t = o inserted),
// each part multiplied by the factor in Fp (measure.cpp:79-93: a copy, then
// `*= factor`, one rounding per part).  A = double applies a double factor
// to complex64 parts and rounds once (the precision form).
template <class T, class A>
__global__ void __launch_bounds__(256) k_compact(const cplx<T> *__restrict__ src,
                                                 cplx<T> *__restrict__ dst, uint64_t ndst, unsigned t,
                                                 unsigned outcome, A factor)
{
    const uint64_t keep = uint64_t(outcome) << t;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < ndst; j += stride) {
        cplx<T> a = src[insert0(j, t) | keep];
        a.x = T(rn<A>::mul(A(a.x), factor));
        a.y = T(rn<A>::mul(A(a.y), factor));
        dst[j] = a;
    }
}

int alloc_raw(qslc_state *s, uint64_t count, void **out)
{
    *out = nullptr;
    cudaError_t e = cudaMalloc(out, count * s->amp_bytes());
    if (e != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return fail(QSLC_EOOM, "out of device memory for " + std::to_string(count) + " amplitudes");
    }
    return QSLC_OK;
}

// Replace the amplitude array by `p` holding `cap` amplitudes; the old one is
// freed once the work queued on the handle's stream has finished with it.
int swap_buffer(qslc_state *s, void *p, uint64_t cap)
{
    cudaError_t e = cudaStreamSynchronize(s->stream);
    cudaFree(s->amps);
    s->amps = p;
    s->cap = cap;
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    return QSLC_OK;
}

}  // namespace

int resize_add_qubit(qslc_state *s, unsigned targ)
{
    const uint64_t dim = s->namps;
    const uint64_t grid = grid_for(dim);
    const void *src = s->amps;
    void *dst = s->amps;
    void *fresh = nullptr;
    if (2 * dim > s->cap) {
        // no room: the reference doubles its storage (resize.cpp:111-118)
        int rc = alloc_raw(s, 2 * dim, &fresh);
        if (rc) return rc;
        dst = fresh;
    } else {
        int rc = s->scratch2.ensure(dim * s->amp_bytes());
        if (rc) return rc;
        QSLC_CUDA(cudaMemcpyAsync(s->scratch2.ptr, s->amps, dim * s->amp_bytes(),
                                  cudaMemcpyDeviceToDevice, s->stream));
        src = s->scratch2.ptr;
    }
    if (s->dtype == QSLC_C128)
        k_expand<double><<<unsigned(grid), 256, 0, s->stream>>>(static_cast<const double2 *>(src),
                                                                static_cast<double2 *>(dst), dim, targ);
    else
        k_expand<float><<<unsigned(grid), 256, 0, s->stream>>>(static_cast<const float2 *>(src),
                                                               static_cast<float2 *>(dst), dim, targ);
    s->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        if (fresh) cudaFree(fresh);
        return cuda_fail(e, "k_expand");
    }
    if (fresh) {
        int rc = swap_buffer(s, fresh, 2 * dim);
        if (rc) return rc;
    }
    s->n += 1;
    s->namps = 2 * dim;
    return QSLC_OK;
}

int resize_collapse_out(qslc_state *s, unsigned targ, unsigned outcome, double factor, bool f64)
{
    const uint64_t half = s->namps / 2;
    int rc = s->scratch2.ensure(half * s->amp_bytes());
    if (rc) return rc;
    const unsigned grid = grid_for(half);
    if (s->dtype == QSLC_C128)
        k_compact<double, double><<<grid, 256, 0, s->stream>>>(
            static_cast<const double2 *>(s->amps), static_cast<double2 *>(s->scratch2.ptr), half, targ,
            outcome, factor);
    else if (f64)
        k_compact<float, double><<<grid, 256, 0, s->stream>>>(
            static_cast<const float2 *>(s->amps), static_cast<float2 *>(s->scratch2.ptr), half, targ,
            outcome, factor);
    else
        k_compact<float, float><<<grid, 256, 0, s->stream>>>(
            static_cast<const float2 *>(s->amps), static_cast<float2 *>(s->scratch2.ptr), half, targ,
            outcome, float(factor));
    s->launches++;
    QSLC_CUDA(cudaGetLastError());
    QSLC_CUDA(cudaMemcpyAsync(s->amps, s->scratch2.ptr, half * s->amp_bytes(), cudaMemcpyDeviceToDevice,
                              s->stream));
    s->n -= 1;
    s->namps = half;
    return QSLC_OK;
}

int resize_reallocate(qslc_state *s)
{
    if (s->cap == s->namps) return QSLC_OK;
    void *fresh = nullptr;
    int rc = alloc_raw(s, s->namps, &fresh);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(fresh, s->amps, s->namps * s->amp_bytes(), cudaMemcpyDeviceToDevice,
                                    s->stream);
    if (e != cudaSuccess) {
        cudaFree(fresh);
        return cuda_fail(e, "reallocate copy");
    }
    return swap_buffer(s, fresh, s->namps);
}

int resize_capacity(qslc_state *s, uint64_t count)
{
    if (count <= s->cap) return QSLC_OK;
    void *fresh = nullptr;
    int rc = alloc_raw(s, count, &fresh);
    if (rc) return rc;
    return swap_buffer(s, fresh, count);
}

}  // namespace qslc
