// fused_tc.cu -- five-qubit dense blocks on the 5th-generation tensor cores.
//
// A fused block U (32 x 32 complex) applied to every group of 32 amplitudes
// is the matrix product D = A * B^T with
//   A [groups x 64]  one row per group: its amplitudes as (re, im) pairs,
//   B [64 x 64]      the real form of U: B[2o+c][2v+d] from U[o][v],
//   D [groups x 64]  the new amplitudes, (re, im) pairs again.
// A CTA takes 128 groups per tile (M = 128), N = 64, K = 64, and issues
// tcgen05.mma kind::tf32 from one thread with the fp32 accumulator in
// tensor memory.  FP32 accuracy comes from the 3xTF32 split: every operand
// x = hi + lo with hi, lo TF32, and D = A_hi B_hi + A_hi B_lo + A_lo B_hi
// (the A_lo B_lo term is below FP32 resolution).
//
// Shared-memory operands use the canonical K-major layout without swizzle:
// core matrices of 8 rows x 16 bytes, 128 contiguous bytes each, ordered
// K-chunk fastest then 8-row group; the descriptors' leading byte offset is
// the step between K-adjacent core matrices (128 B) and the stride byte
// offset the step between 8-row groups (K/4 * 128 B).
//
// Every wait is bounded: if the MMA completion never arrives the kernel
// records an error code, releases its tensor memory and returns.
#include "qslc_internal.cuh"

#include <cstring>
#include <vector>

namespace qslc {
namespace {

constexpr int TC_M = 128;   // groups per tile
constexpr int TC_N = 64;
constexpr int TC_K = 64;
constexpr int CORE_BYTES = 128;
constexpr int A_BYTES = TC_M * TC_K * 4;     // 32 KB per split half
constexpr int B_BYTES = TC_N * TC_K * 4;     // 16 KB per split half
constexpr uint32_t TMEM_COLS = 64;
constexpr long long WAIT_LIMIT = 1ll << 26;

__device__ __forceinline__ uint32_t core_offset(int row, int k)
{
    return uint32_t(((row >> 3) * (TC_K / 4) + (k >> 2)) * CORE_BYTES + (row & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr)
{
    const uint32_t lbo = CORE_BYTES, sbo = (TC_K / 4) * CORE_BYTES;
    uint64_t d = 0;
    d |= uint64_t((saddr >> 4) & 0x3FFF);
    d |= uint64_t((lbo >> 4) & 0x3FFF) << 16;
    d |= uint64_t((sbo >> 4) & 0x3FFF) << 32;
    d |= uint64_t(1) << 46;                  // descriptor version of sm_100 tcgen05
    return d;                                // base offset 0, no swizzle
}

// kind::tf32 instruction descriptor: D f32, A/B tf32, both K-major, N, M
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(TC_N >> 3) << 17) |
                           (uint32_t(TC_M >> 4) << 24);

__device__ __forceinline__ uint32_t to_tf32(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// TF32 split of four consecutive K entries of one row: x = hi + lo.
__device__ __forceinline__ void split4(float4 x, uint4 &hi, uint4 &lo)
{
    hi = make_uint4(to_tf32(x.x), to_tf32(x.y), to_tf32(x.z), to_tf32(x.w));
    lo = make_uint4(to_tf32(x.x - __uint_as_float(hi.x)), to_tf32(x.y - __uint_as_float(hi.y)),
                    to_tf32(x.z - __uint_as_float(hi.z)), to_tf32(x.w - __uint_as_float(hi.w)));
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t acc)
{
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(IDESC), "r"(acc));
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase)
{
    uint32_t done = 0;
    for (long long it = 0; it < WAIT_LIMIT && !done; it++) {
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(phase));
    }
    return done != 0;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
        "%12, %13, %14, %15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

// bmat: B_hi then B_lo, each [64 n][64 k] row-major fp32 (tf32 values).
//
// Pipeline per tile: the 32 amplitudes of this thread's group wait in
// registers; they are split into shared memory (16-byte stores, one row of
// a core matrix each), one thread issues the MMAs, and while they run every
// thread already loads the next tile's amplitudes into the same registers.
// Tiles cover disjoint groups, so reading the next tile before the current
// one is written back is safe.
__global__ void __launch_bounds__(TC_M) k_dense_tc(float2 *__restrict__ st, uint64_t ngroups,
                                                   const float *__restrict__ bmat, uint4 pos_lo,
                                                   unsigned pos_hi, int *__restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *a_hi = smem, *a_lo = smem + A_BYTES;
    unsigned char *b_hi = smem + 2 * A_BYTES, *b_lo = b_hi + B_BYTES;
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    __shared__ int arrived;
    __shared__ uint64_t s_off[32];
    const int tid = threadIdx.x, warp = tid >> 5;
    const unsigned pos[5] = {pos_lo.x, pos_lo.y, pos_lo.z, pos_lo.w, pos_hi};
    if (tid < 32) {
        uint64_t o = 0;
#pragma unroll
        for (int j = 0; j < 5; j++)
            if (tid & (1 << j)) o |= uint64_t(1) << pos[j];
        s_off[tid] = o;
    }
    // B into the canonical layout (rows n, columns k)
    for (int i = tid; i < TC_N * TC_K; i += TC_M) {
        const int n = i / TC_K, k = i % TC_K;
        const uint32_t o = core_offset(n, k);
        *reinterpret_cast<float *>(b_hi + o) = bmat[i];
        *reinterpret_cast<float *>(b_lo + o) = bmat[TC_N * TC_K + i];
    }
    const uint32_t mbar_s = uint32_t(__cvta_generic_to_shared(&mbar));
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar_s));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (warp == 0) {
        const uint32_t slot = uint32_t(__cvta_generic_to_shared(&tmem_slot));
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_slot;
    const uint32_t a_hi_s = uint32_t(__cvta_generic_to_shared(a_hi));
    const uint32_t a_lo_s = uint32_t(__cvta_generic_to_shared(a_lo));
    const uint32_t b_hi_s = uint32_t(__cvta_generic_to_shared(b_hi));
    const uint32_t b_lo_s = uint32_t(__cvta_generic_to_shared(b_lo));
    const uint64_t ntiles = ngroups / TC_M;
    auto group_base = [&](uint64_t t) {
        uint64_t b = t * TC_M + tid;
#pragma unroll
        for (int j = 0; j < 5; j++) b = insert0(b, pos[j]);
        return b;
    };
    float2 a[32];
    uint64_t t = blockIdx.x;
    if (t < ntiles) {
        const uint64_t b0 = group_base(t);
#pragma unroll
        for (int v = 0; v < 32; v++) a[v] = st[b0 | s_off[v]];
    }
    uint32_t phase = 0;
    bool ok = true;
    for (; t < ntiles && ok; t += gridDim.x) {
        const uint64_t base = group_base(t);
        // row `tid` of A: K entries 4j..4j+3 are amplitudes 2j, 2j+1 as (re, im)
#pragma unroll
        for (int j = 0; j < 16; j++) {
            uint4 hi, lo;
            split4(make_float4(a[2 * j].x, a[2 * j].y, a[2 * j + 1].x, a[2 * j + 1].y), hi, lo);
            const uint32_t o = core_offset(tid, 4 * j);
            *reinterpret_cast<uint4 *>(a_hi + o) = hi;
            *reinterpret_cast<uint4 *>(a_lo + o) = lo;
        }
        asm volatile("fence.proxy.async.shared::cta;");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (tid == 0) {
            uint32_t acc = 0;
#pragma unroll
            for (int s = 0; s < TC_K / 8; s++) {       // K = 8 per instruction: two core matrices
                const uint32_t koff = uint32_t(2 * s * CORE_BYTES);
                mma_tf32(tmem, smem_desc(a_hi_s + koff), smem_desc(b_hi_s + koff), acc);
                acc = 1;
                mma_tf32(tmem, smem_desc(a_hi_s + koff), smem_desc(b_lo_s + koff), 1);
                mma_tf32(tmem, smem_desc(a_lo_s + koff), smem_desc(b_hi_s + koff), 1);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                mbar_s));
        }
        // the next tile's amplitudes travel while the MMAs run
        const uint64_t tn = t + gridDim.x;
        if (tn < ntiles) {
            const uint64_t bn = group_base(tn);
#pragma unroll
            for (int v = 0; v < 32; v++) a[v] = st[bn | s_off[v]];
        }
        // one thread polls the barrier (bounded); the block follows its outcome
        if (tid == 0) arrived = mbar_wait(mbar_s, phase) ? 1 : 0;
        __syncthreads();
        if (!arrived) {
            ok = false;
            if (tid == 0) {
                atomicExch(err, 1);
                mbar_wait(mbar_s, phase);            // give work in flight a last bounded wait
            }
            break;
        }
        phase ^= 1;
        asm volatile("tcgen05.fence::after_thread_sync;");
        // row tid of D: lane tid of tensor memory, 64 fp32 columns
        const uint32_t taddr = tmem + (uint32_t(warp * 32) << 16);
#pragma unroll
        for (int c = 0; c < 4; c++) {
            uint32_t r[16];
            tmem_ld16(taddr + uint32_t(16 * c), r);
            asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const int v = 8 * c + i;
                st[base | s_off[v]] = make_float2(__uint_as_float(r[2 * i]), __uint_as_float(r[2 * i + 1]));
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
    }
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
}

// host: TF32 rounding, to nearest with ties away from zero (cvt.rna)
float tf32_host(float x)
{
    uint32_t b;
    std::memcpy(&b, &x, 4);
    if ((b & 0x7F800000u) != 0x7F800000u) b = (b + 0x1000u) & ~0x1FFFu;
    float r;
    std::memcpy(&r, &b, 4);
    return r;
}

}  // namespace

// B = real form of the 32x32 complex block U (U[o*32+v]), split hi/lo.
void tc_pack_block(const std::vector<cd> &U, float *out)
{
    float *hi = out, *lo = out + TC_N * TC_K;
    for (int o = 0; o < 32; o++)
        for (int v = 0; v < 32; v++) {
            const double ur = U[size_t(o) * 32 + v].real(), ui = U[size_t(o) * 32 + v].imag();
            const double val[2][2] = {{ur, -ui}, {ui, ur}};   // [c_out][c_in]
            for (int co = 0; co < 2; co++)
                for (int ci = 0; ci < 2; ci++) {
                    const float x = float(val[co][ci]);
                    const float h = tf32_host(x);
                    const float l = tf32_host(x - h);
                    const int idx = (2 * o + co) * TC_K + (2 * v + ci);
                    hi[idx] = h;
                    lo[idx] = l;
                }
        }
}

size_t tc_block_floats() { return size_t(2) * TC_N * TC_K; }

bool tc_usable(const qslc_state *s) { return s->n >= 12; }

int tc_launch(qslc_state *s, const float *d_b, const unsigned *pos, int *d_err)
{
    const uint64_t ngroups = uint64_t(1) << (s->n - 5);
    const int smem = 2 * A_BYTES + 2 * B_BYTES;
    static bool attr = false;
    if (!attr) {
        QSLC_CUDA(cudaFuncSetAttribute(k_dense_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr = true;
    }
    const uint64_t tiles = ngroups / TC_M;
    const unsigned grid = unsigned(std::min<uint64_t>(tiles, uint64_t(sm_count()) * 2));
    k_dense_tc<<<grid, TC_M, smem, s->stream>>>(static_cast<float2 *>(s->amps), ngroups, d_b,
                                                make_uint4(pos[0], pos[1], pos[2], pos[3]), pos[4], d_err);
    s->launches++;
    QSLC_CUDA(cudaGetLastError());
    return QSLC_OK;
}

}  // namespace qslc
