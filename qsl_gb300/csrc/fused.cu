// fused.cu -- the precision form: fused dense blocks on complex64 states.
//
// With fusion on (qslc_set_fusion), gates on a complex64 state are queued.
// At the next call that reads or measures the state, the queue is planned
// into blocks of at most k qubits (fusion_host.hpp), each block's 2^k x 2^k
// unitary is built on the host in double precision and rounded to float,
// and one sweep per block applies it.  This trades the reference's
// operation-by-operation rounding for one FP32 matrix-vector product per
// block: amplitudes agree with the FP64 path to about 1e-6 relative
// (infidelity far below 1e-6), and a sweep applies many gates at once.
//
// Kernel: one thread owns one group of 2^k amplitudes -- a base index with
// zeros at the block's qubit positions, plus every combination of those
// bits.  Consecutive threads own consecutive bases, so each of the 2^k
// loads and stores of a warp is one contiguous run of 32 amplitudes
// whenever qubit 0 is outside the block.  The block matrix sits in shared
// memory and every thread reads the same element at the same time
// (broadcast).
#include "fusion_host.hpp"
#include "qslc_internal.cuh"

#include <vector>

namespace qslc {
namespace {

template <int K>
__global__ void __launch_bounds__(256) k_dense(float2 *__restrict__ st, uint64_t ngroups,
                                               const float2 *__restrict__ U, uint4 pos_lo,
                                               unsigned pos_hi)
{
    constexpr int D = 1 << K;
    __shared__ float2 u[D * D];
    for (int i = threadIdx.x; i < D * D; i += blockDim.x) u[i] = U[i];
    __syncthreads();
    const unsigned pos[5] = {pos_lo.x, pos_lo.y, pos_lo.z, pos_lo.w, pos_hi};
    uint64_t off[D];
#pragma unroll
    for (int v = 0; v < D; v++) {
        uint64_t o = 0;
#pragma unroll
        for (int j = 0; j < K; j++)
            if (v & (1 << j)) o |= uint64_t(1) << pos[j];
        off[v] = o;
    }
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t g = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; g < ngroups; g += stride) {
        uint64_t base = g;
#pragma unroll
        for (int j = 0; j < K; j++) base = insert0(base, pos[j]);   // ascending positions
        float2 a[D];
#pragma unroll
        for (int v = 0; v < D; v++) a[v] = st[base | off[v]];
#pragma unroll 4
        for (int o = 0; o < D; o++) {
            float re = 0.f, im = 0.f;
#pragma unroll
            for (int v = 0; v < D; v++) {
                const float2 m = u[o * D + v];
                re = fmaf(m.x, a[v].x, re);
                re = fmaf(-m.y, a[v].y, re);
                im = fmaf(m.x, a[v].y, im);
                im = fmaf(m.y, a[v].x, im);
            }
            st[base | off[o]] = make_float2(re, im);
        }
    }
}

template <int K>
void launch_dense(qslc_state *s, const float2 *U, const unsigned *pos)
{
    const uint64_t ngroups = uint64_t(1) << (s->n - K);
    uint4 lo = make_uint4(K > 0 ? pos[0] : 0, K > 1 ? pos[1] : 0, K > 2 ? pos[2] : 0, K > 3 ? pos[3] : 0);
    const unsigned hi = K > 4 ? pos[4] : 0;
    k_dense<K><<<grid_for(ngroups, 256, 8), 256, 0, s->stream>>>(static_cast<float2 *>(s->amps),
                                                                 ngroups, U, lo, hi);
    s->launches++;
}

}  // namespace

int fusion_flush(qslc_state *s)
{
    if (s->fuse_queue.empty()) return QSLC_OK;
    std::vector<Block> blocks = plan_blocks(s->fuse_queue, int(s->fuse_k < 2 ? 2 : s->fuse_k), s->n);
    s->fuse_queue.clear();
    size_t total = 0;
    for (const Block &b : blocks) total += size_t(1) << (2 * b.k);
    std::vector<float2> mats(total);
    size_t at = 0;
    for (const Block &b : blocks) {
        const size_t cnt = size_t(1) << (2 * b.k);
        for (size_t i = 0; i < cnt; i++) mats[at + i] = make_float2(float(b.U[i].real()), float(b.U[i].imag()));
        at += cnt;
    }
    int rc = s->fuse_mats.ensure(total * sizeof(float2));
    if (rc) return rc;
    float2 *d = static_cast<float2 *>(s->fuse_mats.ptr);
    QSLC_CUDA(cudaMemcpyAsync(d, mats.data(), total * sizeof(float2), cudaMemcpyHostToDevice, s->stream));
    // five-qubit blocks for the tensor cores: their real-form operands, split
    const bool tc = s->fuse_tc && tc_usable(s);
    float *d_tc = nullptr;
    int *d_err = nullptr;
    std::vector<float> packed;
    if (tc) {
        size_t n5 = 0;
        for (const Block &b : blocks) n5 += b.k == 5;
        const size_t per = tc_block_floats();
        packed.resize(n5 * per + 4);
        size_t i5 = 0;
        for (const Block &b : blocks)
            if (b.k == 5) tc_pack_block(b.U, packed.data() + per * i5++);
        rc = s->fuse_tc_mats.ensure(packed.size() * sizeof(float));
        if (rc) return rc;
        d_tc = static_cast<float *>(s->fuse_tc_mats.ptr);
        d_err = reinterpret_cast<int *>(d_tc + n5 * per);
        QSLC_CUDA(cudaMemcpyAsync(d_tc, packed.data(), packed.size() * sizeof(float), cudaMemcpyHostToDevice,
                                  s->stream));
        QSLC_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), s->stream));
    }
    at = 0;
    size_t i5 = 0;
    for (const Block &b : blocks) {
        const float2 *U = d + at;
        if (tc && b.k == 5) {
            rc = tc_launch(s, d_tc + tc_block_floats() * i5++, b.qubits, d_err);
            if (rc) return rc;
            at += size_t(1) << (2 * b.k);
            s->fused_blocks++;
            continue;
        }
        switch (b.k) {
        case 1: launch_dense<1>(s, U, b.qubits); break;
        case 2: launch_dense<2>(s, U, b.qubits); break;
        case 3: launch_dense<3>(s, U, b.qubits); break;
        case 4: launch_dense<4>(s, U, b.qubits); break;
        default: launch_dense<5>(s, U, b.qubits); break;
        }
        at += size_t(1) << (2 * b.k);
        s->fused_blocks++;
    }
    // a copy from pageable memory has left `mats` once cudaMemcpyAsync returns
    QSLC_CUDA(cudaGetLastError());
    if (tc) {
        int err = 0;
        QSLC_CUDA(cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
        QSLC_CUDA(cudaStreamSynchronize(s->stream));
        if (err) return fail(QSLC_ETIMEOUT, "a tensor-core block did not complete in time");
    }
    return QSLC_OK;
}

}  // namespace qslc
