// gates.cu -- amplitude-pair sweeps of the plain (2^n) layout.
//
// The sweeps: k_pair1 / k_diag1 / k_pair2 / k_diag2, one gate per sweep
// from registers; k_group2, two one-qubit gates on different qubits in one
// sweep; k_pair1_shfl, pairs inside a warp exchanged between lanes; and
// the staged sweeps through shared memory (opt-in, stage.cuh).
//
// One thread owns one amplitude pair (or one amplitude for the diagonal
// gates) in a grid-stride loop.  The pair index j is turned into the basis
// index by inserting the target bit (bit insertion replaces the reference's
// nested s/r loops, gates.cpp:36-37, and its triple i/j/k loops for two
// qubits, :227-231); consecutive threads touch consecutive 16-byte
// amplitudes, so every warp reads and writes whole 32-byte sectors for any
// target above 0.
//
// Arithmetic is the reference's, operation for operation, with no
// contraction into FMA: the x86-64 reference rounds each product and each
// sum, and so does every update below (rn<T>::mul/add/sub/div).
#include "qslc_internal.cuh"
#include "gatemath.cuh"
#include "stage.cuh"

#include <cmath>
#include <cstdlib>
#include <utility>
#include <vector>

namespace qslc {
namespace {

// Debug builds (-DQSLC_DEBUG_BOUNDS) check each item's largest index
// against the state's size before the item is read or written: an index
// outside the state is recorded (the first one) and the item skipped, and
// the next call that reads the state returns QSLC_EINVAL with the index
// (debug_bounds_error).  The host validates every qubit index before a
// launch, so no call through the ABI should record one.  Default builds
// compile both checks to `true`.
#ifdef QSLC_DEBUG_BOUNDS
__device__ unsigned long long g_bad_index;   // first index outside a state, plus one; 0: none
__device__ __forceinline__ bool in_state(uint64_t i, uint64_t dim)
{
    if (i < dim) return true;
    atomicCAS(&g_bad_index, 0ull, (unsigned long long)i + 1ull);
    return false;
}
#define QSLC_IN_STATE(i, dim) in_state(uint64_t(i), uint64_t(dim))
#define QSLC_IN_STATE_QUIET(i, dim) (uint64_t(i) < uint64_t(dim))
#else
#define QSLC_IN_STATE(i, dim) true
#define QSLC_IN_STATE_QUIET(i, dim) true
#endif


// One-qubit pair gates: pairs (i0, i0 + 2^t), i0 = insert0(j, t).
template <class T, int OP, unsigned CPAT = PAT_RUNTIME, class IX = uint64_t>
__global__ void QSLC_SWEEP_BOUNDS k_pair1(cplx<T> *__restrict__ st, uint64_t npairs,
                                               unsigned t, Coef<T> k, unsigned pat)
{
    const IX bit = IX(1) << t;
    const IX stride = IX(gridDim.x) * blockDim.x;
    const unsigned pt = CPAT == PAT_RUNTIME ? pat : CPAT;
    for (IX j = IX(blockIdx.x) * blockDim.x + threadIdx.x; j < IX(npairs); j += ITEMS * stride) {
        cplx<T> a0[ITEMS], a1[ITEMS];
        IX i0[ITEMS];
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            i0[r] = ins0<IX>(j + r * stride, t);
            if (j + r * stride < npairs && QSLC_IN_STATE(i0[r] | bit, 2 * npairs)) {
                a0[r] = st[i0[r]];
                a1[r] = st[i0[r] | bit];
            }
        }
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            if (j + r * stride < npairs && QSLC_IN_STATE_QUIET(i0[r] | bit, 2 * npairs)) {
                pair_update<T, OP>(a0[r], a1[r], k, (pt >> (8 * r)) & 0xFFu);
                st[i0[r]] = a0[r];
                st[i0[r] | bit] = a1[r];
            }
        }
    }
}

// x with its sign bit XORed with bit 31 of `m` (an exact negation when set);
// integer operations, so a per-lane choice of sign never becomes a branch.
__device__ __forceinline__ double flip_sign(double x, uint32_t m)
{
    return __hiloint2double(__double2hiint(x) ^ int(m), __double2loint(x));
}
__device__ __forceinline__ float flip_sign(float x, uint32_t m)
{
    return __int_as_float(__float_as_int(x) ^ int(m));
}
// x when m is 0, y when m is all ones, by bit operations.
__device__ __forceinline__ double pick(double x, double y, uint32_t m)
{
    const int hi = (__double2hiint(x) & ~int(m)) | (__double2hiint(y) & int(m));
    const int lo = (__double2loint(x) & ~int(m)) | (__double2loint(y) & int(m));
    return __hiloint2double(hi, lo);
}
__device__ __forceinline__ float pick(float x, float y, uint32_t m)
{
    return __int_as_float((__float_as_int(x) & ~int(m)) | (__float_as_int(y) & int(m)));
}

// One output pair of a one-qubit pair gate, computed by the lane that holds
// amplitude `a` (side 0: a = a0, side 1: a = a1) from its partner `o`.  Each
// output is the same RN(p1 +- p2) of the same products as in pair_update:
// the lane's side is folded into exact sign flips (x - y == x + (-y),
// RN(-x) == -RN(x)) and the order of a sum's two terms (they commute), so
// every lane of a warp runs the same instructions.  `m1` is 0x80000000 on
// side 1 and 0 on side 0, `m0` the opposite.  Modes E0, E1 of `md` apply to
// the lane's x and y outputs.
//
// Hadamard's side 1 takes its difference as a0 + (-a1) with the terms
// swapped in, not as a negated a1 - a0: the two differ in the sign of an
// exact zero.
template <class T, int OP>
__device__ __forceinline__ void lane_update(cplx<T> &a, const cplx<T> &o, uint32_t m0, uint32_t m1,
                                            const Coef<T> &k, unsigned md)
{
    const unsigned E0 = mode_of(md, 0), E1 = mode_of(md, 1);
    cplx<T> r;
    if constexpr (OP == P_SWAP) {
        r = o;
    } else if constexpr (OP == P_Y) {        // side 0: (a1.y, -a1.x); side 1: (-a0.y, a0.x)
        r.x = flip_sign(o.y, m1);
        r.y = flip_sign(o.x, m0);
    } else if constexpr (OP == P_H) {        // side 0: (a0 + a1)/r; side 1: (a0 + (-a1))/r
        const uint32_t all = uint32_t(int32_t(m1) >> 31);
        r.x = hdiv<T, false>(E0 != MD_F, pick(a.x, o.x, all), flip_sign(pick(o.x, a.x, all), m1), k);
        r.y = hdiv<T, false>(E1 != MD_F, pick(a.y, o.y, all), flip_sign(pick(o.y, a.y, all), m1), k);
    } else if constexpr (OP == P_RX) {       // the same on both sides
        r.x = dot2m<T, false>(E0, a.x, k.c, k.kc, k.mc, o.y, k.s, k.ks, k.ms);
        r.y = dot2m<T, true>(E1, a.y, k.c, k.kc, k.mc, o.x, k.s, k.ks, k.ms);
    } else if constexpr (OP == P_RY) {       // side 0: a0 c - a1 s; side 1: a1 c + a0 s
        r.x = dot2m<T, false>(E0, a.x, k.c, k.kc, k.mc, flip_sign(o.x, m0), k.s, k.ks, k.ms);
        r.y = dot2m<T, false>(E1, a.y, k.c, k.kc, k.mc, flip_sign(o.y, m0), k.s, k.ks, k.ms);
    } else {                                 // P_RZ, no partner: side 1 flips the sign of s
        r.x = dot2m<T, false>(E0, a.x, k.c, k.kc, k.mc, flip_sign(a.y, m1), k.s, k.ks, k.ms);
        r.y = dot2m<T, true>(E1, a.y, k.c, k.kc, k.mc, flip_sign(a.x, m1), k.s, k.ks, k.ms);
    }
    a = r;
}

// One-qubit pair gates on targets 0-4 as warp exchanges (QSLC_SHFL=1).  A
// pair (i, i ^ 2^t) then lies within 32 consecutive amplitudes: lane l of a
// warp holds amplitude base + l, so a warp loads and stores 512 contiguous
// bytes per item, and takes its partner's amplitude from lane l ^ 2^t with
// shuffles.  A lane holds 2 ITEMS amplitudes per iteration, the register
// sweep's ITEMS pairs; item 2r takes modes E0, E1 of the pattern's item r,
// item 2r + 1 its E2, E3, so the split between the pipes is the same.
// `namps` is a multiple of 32 and the stride a multiple of the block, so
// the loop bound and every item test are the same across a warp, and the
// shuffles always run with all 32 lanes.
template <class T, int OP, unsigned CPAT = PAT_RUNTIME, class IX = uint64_t>
__global__ void QSLC_SWEEP_BOUNDS k_pair1_shfl(cplx<T> *__restrict__ st, uint64_t namps, unsigned t,
                                                Coef<T> k, unsigned pat)
{
    constexpr int N = 2 * ITEMS;
    const IX stride = IX(gridDim.x) * blockDim.x;
    const unsigned pt = CPAT == PAT_RUNTIME ? pat : CPAT;
    const unsigned lanebit = 1u << t;
    const uint32_t m1 = (threadIdx.x & lanebit) ? 0x80000000u : 0u, m0 = m1 ^ 0x80000000u;
    for (IX i = IX(blockIdx.x) * blockDim.x + threadIdx.x; i < IX(namps); i += N * stride) {
        cplx<T> a[N];
#pragma unroll
        for (int r = 0; r < N; r++)
            if (i + r * stride < namps) a[r] = st[i + r * stride];
#pragma unroll
        for (int r = 0; r < N; r++) {
            if (i + r * stride < namps) {
                cplx<T> o = a[r];
                if constexpr (OP != P_RZ) {
                    o.x = __shfl_xor_sync(0xFFFFFFFFu, a[r].x, lanebit);
                    o.y = __shfl_xor_sync(0xFFFFFFFFu, a[r].y, lanebit);
                }
                lane_update<T, OP>(a[r], o, m0, m1, k, ((pt >> (8 * (r >> 1))) >> (4 * (r & 1))) & 0xFu);
                st[i + r * stride] = a[r];
            }
        }
    }
}

// One-qubit diagonal gates on the |1> half: index insert0(j, t) | 2^t.
template <class T, int OP, unsigned CPAT = PAT_RUNTIME, class IX = uint64_t>
__global__ void QSLC_SWEEP_BOUNDS k_diag1(cplx<T> *__restrict__ st, uint64_t count,
                                               unsigned t, Coef<T> k, unsigned pat)
{
    const IX bit = IX(1) << t;
    const IX stride = IX(gridDim.x) * blockDim.x;
    const unsigned pt = CPAT == PAT_RUNTIME ? pat : CPAT;
    for (IX j = IX(blockIdx.x) * blockDim.x + threadIdx.x; j < IX(count); j += ITEMS * stride) {
        cplx<T> a[ITEMS];
        IX i[ITEMS];
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            i[r] = ins0<IX>(j + r * stride, t) | bit;
            if (j + r * stride < count && QSLC_IN_STATE(i[r], 2 * count)) a[r] = st[i[r]];
        }
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            if (j + r * stride < count && QSLC_IN_STATE_QUIET(i[r], 2 * count)) {
                diag_update<T, OP>(a[r], k, (pt >> (8 * r)) & 0xFFu);
                st[i[r]] = a[r];
            }
        }
    }
}

// Two one-qubit gates on different qubits in one sweep (gate grouping).
// A thread holds the four amplitudes that differ only in the two target
// bits, applies the first gate to its two pairs along the first gate's bit
// and then the second gate to its two pairs along the other bit.  Every
// amplitude sees the same operations, in the same order, as in two
// sweeps, so the bits are those of the two gates one after the other; the
// state is read and written once instead of twice.
//
// `op` is a PairOp, or GROUP_DIAG + a DiagOp for phase and pauliZ (which
// act on the members with the bit set).  The output modes (gatemath.cuh)
// are fixed per gate type: the two pair updates of a rotation take the
// low and high byte of QSLC_GROUP_MODES_ROT, and so on.
constexpr int GROUP_DIAG = 16;
#ifndef QSLC_GROUP_MODES_ROT
#define QSLC_GROUP_MODES_ROT 0x1595u      // PPPQ, PPPF
#endif
#ifndef QSLC_GROUP_MODES_H
#define QSLC_GROUP_MODES_H 0x0000u        // FFFF, FFFF
#endif
#ifndef QSLC_GROUP_MODES_DIAG
#define QSLC_GROUP_MODES_DIAG 0x0509u     // PQ, PP
#endif

template <class T>
struct GroupGates {
    int op[2];
    Coef<T> k[2];
};

// One gate of a group on the pairs (x0, x1) and (y0, y1); x1 and y1 are
// the members with the gate's bit set.
template <class T>
__device__ __forceinline__ void group_apply(int op, cplx<T> &x0, cplx<T> &x1, cplx<T> &y0, cplx<T> &y1,
                                            const Coef<T> &k)
{
    constexpr unsigned R0 = QSLC_GROUP_MODES_ROT & 0xFFu, R1 = (QSLC_GROUP_MODES_ROT >> 8) & 0xFFu;
    constexpr unsigned H0 = QSLC_GROUP_MODES_H & 0xFFu, H1 = (QSLC_GROUP_MODES_H >> 8) & 0xFFu;
    constexpr unsigned D0 = QSLC_GROUP_MODES_DIAG & 0xFFu, D1 = (QSLC_GROUP_MODES_DIAG >> 8) & 0xFFu;
    switch (op) {
    case P_SWAP:
        pair_update<T, P_SWAP>(x0, x1, k);
        pair_update<T, P_SWAP>(y0, y1, k);
        break;
    case P_Y:
        pair_update<T, P_Y>(x0, x1, k);
        pair_update<T, P_Y>(y0, y1, k);
        break;
    case P_H:
        pair_update<T, P_H>(x0, x1, k, H0);
        pair_update<T, P_H>(y0, y1, k, H1);
        break;
    case P_RX:
        pair_update<T, P_RX>(x0, x1, k, R0);
        pair_update<T, P_RX>(y0, y1, k, R1);
        break;
    case P_RY:
        pair_update<T, P_RY>(x0, x1, k, R0);
        pair_update<T, P_RY>(y0, y1, k, R1);
        break;
    case P_RZ:
        pair_update<T, P_RZ>(x0, x1, k, R0);
        pair_update<T, P_RZ>(y0, y1, k, R1);
        break;
    case GROUP_DIAG + D_NEG:
        diag_update<T, D_NEG>(x1, k);
        diag_update<T, D_NEG>(y1, k);
        break;
    default:                                  // GROUP_DIAG + D_PHASE
        diag_update<T, D_PHASE>(x1, k, D0);
        diag_update<T, D_PHASE>(y1, k, D1);
        break;
    }
}

// quads j in [0, 2^(n-2)): x = j with zeros inserted at bits lo < hi; the
// first gate acts on bit mask c0, the second on c1 ({c0, c1} = {2^lo, 2^hi}).
template <class T, class IX = uint64_t>
__global__ void QSLC_SWEEP_BOUNDS k_group2(cplx<T> *__restrict__ st, uint64_t nquads, unsigned lo, unsigned hi,
                                                IX c0, IX c1, GroupGates<T> g)
{
    const IX stride = IX(gridDim.x) * blockDim.x;
    for (IX j = IX(blockIdx.x) * blockDim.x + threadIdx.x; j < IX(nquads); j += stride) {
        const IX x = ins00<IX>(j, lo, hi);
        if (!QSLC_IN_STATE(x | c0 | c1, 4 * nquads)) continue;
        cplx<T> a00 = st[x], a01 = st[x | c0], a10 = st[x | c1], a11 = st[x | c0 | c1];
        group_apply<T>(g.op[0], a00, a01, a10, a11, g.k[0]);
        group_apply<T>(g.op[1], a00, a10, a01, a11, g.k[1]);
        st[x] = a00;
        st[x | c0] = a01;
        st[x | c1] = a10;
        st[x | c0 | c1] = a11;
    }
}

// rotateZ touches both halves with different coefficients; it is a pair
// gate whose two members do not mix (gates.cpp:181-209).

// Two-qubit gates: j in [0, 2^(n-2)), base = j with zeros inserted at lo < hi.
// MODE 0: controlled pair (base|b1, base|b1|b2), b1 = control bit;
// MODE 1: number-preserving pair (base|b1, base|b2);
// MODE 2: fswap = MODE 1 swap plus negation of base|b1|b2.
template <class T, int OP, int MODE, unsigned CPAT = PAT_RUNTIME, class IX = uint64_t>
__global__ void QSLC_SWEEP_BOUNDS k_pair2(cplx<T> *__restrict__ st, uint64_t nquads,
                                               unsigned lo, unsigned hi, uint64_t b1,
                                               uint64_t b2, Coef<T> k, unsigned pat)
{
    const IX stride = IX(gridDim.x) * blockDim.x;
    const unsigned pt = CPAT == PAT_RUNTIME ? pat : CPAT;
    for (IX j = IX(blockIdx.x) * blockDim.x + threadIdx.x; j < IX(nquads); j += ITEMS * stride) {
        cplx<T> a0[ITEMS], a1[ITEMS];
        IX x1[ITEMS], x2[ITEMS];
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            const IX base = ins00<IX>(j + r * stride, lo, hi);
            x1[r] = base | IX(b1);
            x2[r] = (MODE == 0) ? (x1[r] | IX(b2)) : (base | IX(b2));
            if (j + r * stride < nquads && QSLC_IN_STATE(x1[r] | IX(b2), 4 * nquads)) {
                a0[r] = st[x1[r]];
                a1[r] = st[x2[r]];
            }
        }
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            if (j + r * stride < nquads && QSLC_IN_STATE_QUIET(x1[r] | IX(b2), 4 * nquads)) {
                pair_update<T, OP>(a0[r], a1[r], k, (pt >> (8 * r)) & 0xFFu);
                st[x1[r]] = a0[r];
                st[x2[r]] = a1[r];
                if constexpr (MODE == 2) {
                    const IX x3 = x1[r] | IX(b2);
                    cplx<T> a = st[x3];
                    diag_update<T, D_NEG>(a, k);
                    st[x3] = a;
                }
            }
        }
    }
}

// controlZ / controlPhase: the |11> quarter (gates.cpp:277-301, :436-465).
template <class T, int OP, unsigned CPAT = PAT_RUNTIME, class IX = uint64_t>
__global__ void QSLC_SWEEP_BOUNDS k_diag2(cplx<T> *__restrict__ st, uint64_t nquads,
                                               unsigned lo, unsigned hi, uint64_t both,
                                               Coef<T> k, unsigned pat)
{
    const IX stride = IX(gridDim.x) * blockDim.x;
    const unsigned pt = CPAT == PAT_RUNTIME ? pat : CPAT;
    for (IX j = IX(blockIdx.x) * blockDim.x + threadIdx.x; j < IX(nquads); j += ITEMS * stride) {
        cplx<T> a[ITEMS];
        IX i[ITEMS];
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            i[r] = ins00<IX>(j + r * stride, lo, hi) | IX(both);
            if (j + r * stride < nquads && QSLC_IN_STATE(i[r], 4 * nquads)) a[r] = st[i[r]];
        }
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            if (j + r * stride < nquads && QSLC_IN_STATE_QUIET(i[r], 4 * nquads)) {
                diag_update<T, OP>(a[r], k, (pt >> (8 * r)) & 0xFFu);
                st[i[r]] = a[r];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Warp-tiled sweeps staged through shared memory (complex128 states of up
// to 31 qubits with at least one tile).  A warp-tile is BULK_PAIRS
// consecutive pair indices j (for the diagonal sweep, BULK_PAIRS touched
// amplitudes), BULK_PPL per lane: for a target t >= BULK_LOG2 its members
// form two runs of BULK_PAIRS consecutive amplitudes 2^t apart, for a lower
// target one run of 2 BULK_PAIRS.  Lane 0 of each warp keeps BULK_DEPTH tiles
// in flight as bulk copies into the warp's buffers; the lanes read their
// pairs from shared memory, the buffer is re-armed with the tile BULK_DEPTH
// ahead, and the lanes compute and store straight to global memory.  Warps
// take tiles w, w + W, w + 2W, ... (W warps in the grid), so a persistent
// grid of a few CTAs per SM sweeps the state with no block-wide
// synchronisation.
//
// A barrier wait that runs out sets *err, waits (bounded) for the copies the
// warp still has in flight, and the warp stops; the host reports
// QSLC_ETIMEOUT at its next synchronising call.
// ---------------------------------------------------------------------------
#ifndef QSLC_BULK_WARPS
#define QSLC_BULK_WARPS 8
#endif
#ifndef QSLC_BULK_DEPTH
#define QSLC_BULK_DEPTH 2
#endif
#ifndef QSLC_BULK_CTAS
#define QSLC_BULK_CTAS 3
#endif
#ifndef QSLC_BULK_PPL_LOG2
#define QSLC_BULK_PPL_LOG2 2
#endif
constexpr int BULK_WARPS = QSLC_BULK_WARPS;        // warps per CTA
constexpr int BULK_DEPTH = QSLC_BULK_DEPTH;        // buffers (tiles in flight) per warp
constexpr int BULK_CTAS_PER_SM = QSLC_BULK_CTAS;
constexpr int BULK_PPL = 1 << QSLC_BULK_PPL_LOG2;  // pairs per lane per tile
constexpr int BULK_LOG2 = 5 + QSLC_BULK_PPL_LOG2;  // log2 of the pairs per warp-tile
constexpr int BULK_PAIRS = 1 << BULK_LOG2;         // pairs per warp-tile
constexpr int BULK_AMPS = 2 * BULK_PAIRS;          // amplitudes a buffer holds

template <class T>
constexpr size_t bulk_smem_bytes()
{
    return size_t(BULK_WARPS) * BULK_DEPTH * BULK_AMPS * sizeof(cplx<T>);
}

// On a timed-out wait at tile index i: record it, then give the copies of
// tiles i .. i+BULK_DEPTH-1 (the ones this warp issued) a bounded wait.
__device__ __forceinline__ void bulk_abort(uint64_t (&bars)[BULK_WARPS][BULK_DEPTH], unsigned warp, uint32_t i,
                                           uint32_t tile, uint32_t W, uint32_t ntiles, int *err)
{
    atomicExch(err, 1);
    for (uint32_t d = 0; d < BULK_DEPTH; d++) {
        const uint32_t ii = i + d;
        if (tile + d * W < ntiles) mbar_wait_bounded(smem_addr(&bars[warp][ii % BULK_DEPTH]), (ii / BULK_DEPTH) & 1);
    }
}

template <class T, int OP, unsigned CPAT = PAT_RUNTIME>
__global__ void __launch_bounds__(BULK_WARPS * 32, BULK_CTAS_PER_SM) k_pair1_bulk(cplx<T> *__restrict__ st, uint32_t ntiles,
                                                                unsigned t, Coef<T> k, unsigned pat, int *err)
{
    extern __shared__ __align__(128) unsigned char bulk_smem[];
    __shared__ __align__(8) uint64_t bars[BULK_WARPS][BULK_DEPTH];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    cplx<T> *buf = reinterpret_cast<cplx<T> *>(bulk_smem) + size_t(warp) * BULK_DEPTH * BULK_AMPS;
    const uint32_t W = gridDim.x * BULK_WARPS;
    const uint32_t w0 = blockIdx.x * BULK_WARPS + warp;
    const unsigned pt = CPAT == PAT_RUNTIME ? pat : CPAT;
    const bool wide = t >= BULK_LOG2;
    const uint32_t bit = 1u << t;
    constexpr uint32_t TILE_BYTES = BULK_AMPS * sizeof(cplx<T>);
    auto first_amp = [&](uint32_t tile) -> uint32_t {
        const uint32_t j0 = tile * BULK_PAIRS;
        return wide ? ins0<uint32_t>(j0, t) : 2 * j0;
    };
    auto issue = [&](uint32_t tile, int s) {
        const uint32_t mb = smem_addr(&bars[warp][s]);
        const uint32_t dst = smem_addr(buf + s * BULK_AMPS);
        const uint32_t a = first_amp(tile);
        mbar_arrive_expect(mb, TILE_BYTES);
        if (wide) {
            bulk_g2s(dst, st + a, TILE_BYTES / 2, mb);
            bulk_g2s(dst + TILE_BYTES / 2, st + a + bit, TILE_BYTES / 2, mb);
        } else {
            bulk_g2s(dst, st + a, TILE_BYTES, mb);
        }
    };
    if (lane == 0) {
        for (int s = 0; s < BULK_DEPTH; s++) mbar_init(smem_addr(&bars[warp][s]), 1);
        mbar_init_fence();
        for (int s = 0; s < BULK_DEPTH; s++)
            if (w0 + s * W < ntiles) issue(w0 + s * W, s);
    }
    __syncwarp();
    uint32_t i = 0;
    for (uint32_t tile = w0; tile < ntiles; tile += W, i++) {
        const int s = int(i % BULK_DEPTH);
        int ok = 1;
        if (lane == 0) ok = mbar_wait_bounded(smem_addr(&bars[warp][s]), (i / BULK_DEPTH) & 1) ? 1 : 0;
        ok = __shfl_sync(0xFFFFFFFFu, ok, 0);
        if (!ok) {
            if (lane == 0) bulk_abort(bars, warp, i, tile, W, ntiles, err);
            return;
        }
        const cplx<T> *b = buf + s * BULK_AMPS;
        cplx<T> a0[BULK_PPL], a1[BULK_PPL];
        uint32_t loc[BULK_PPL];
#pragma unroll
        for (int q = 0; q < BULK_PPL; q++) {
            const uint32_t p = lane + 32 * q;
            loc[q] = wide ? p : ins0<uint32_t>(p, t);
            a0[q] = b[loc[q]];
            a1[q] = b[wide ? BULK_PAIRS + p : loc[q] + bit];
        }
        __syncwarp();
        if (lane == 0) {
            fence_proxy_async_smem();
            if (tile + BULK_DEPTH * W < ntiles) issue(tile + BULK_DEPTH * W, s);
        }
        const uint32_t a = first_amp(tile);
#pragma unroll
        for (int q = 0; q < BULK_PPL; q++) {
            pair_update<T, OP>(a0[q], a1[q], k, (pt >> (8 * (q % 3))) & 0xFFu);
            const uint32_t x0 = a + loc[q];
            st[x0] = a0[q];
            st[x0 + bit] = a1[q];
        }
    }
}

// The diagonal sweep (phase, pauliZ) over the |1> half: a warp-tile is the
// BULK_PAIRS amplitudes insert0(j, t) | 2^t of BULK_PAIRS consecutive j --
// one run of them for t >= BULK_LOG2; for a lower target every other run of
// 2^t in a region of 2 BULK_PAIRS amplitudes, which the tile copies whole.
template <class T, int OP, unsigned CPAT = PAT_RUNTIME>
__global__ void __launch_bounds__(BULK_WARPS * 32, BULK_CTAS_PER_SM) k_diag1_bulk(cplx<T> *__restrict__ st, uint32_t ntiles,
                                                                unsigned t, Coef<T> k, unsigned pat, int *err)
{
    extern __shared__ __align__(128) unsigned char bulk_smem[];
    __shared__ __align__(8) uint64_t bars[BULK_WARPS][BULK_DEPTH];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    cplx<T> *buf = reinterpret_cast<cplx<T> *>(bulk_smem) + size_t(warp) * BULK_DEPTH * BULK_AMPS;
    const uint32_t W = gridDim.x * BULK_WARPS;
    const uint32_t w0 = blockIdx.x * BULK_WARPS + warp;
    const unsigned pt = CPAT == PAT_RUNTIME ? pat : CPAT;
    const bool wide = t >= BULK_LOG2;
    const uint32_t bit = 1u << t;
    const uint32_t bytes = (wide ? BULK_PAIRS : BULK_AMPS) * uint32_t(sizeof(cplx<T>));
    auto first_amp = [&](uint32_t tile) -> uint32_t {
        const uint32_t j0 = tile * BULK_PAIRS;
        return wide ? (ins0<uint32_t>(j0, t) | bit) : 2 * j0;
    };
    auto issue = [&](uint32_t tile, int s) {
        const uint32_t mb = smem_addr(&bars[warp][s]);
        mbar_arrive_expect(mb, bytes);
        bulk_g2s(smem_addr(buf + s * BULK_AMPS), st + first_amp(tile), bytes, mb);
    };
    if (lane == 0) {
        for (int s = 0; s < BULK_DEPTH; s++) mbar_init(smem_addr(&bars[warp][s]), 1);
        mbar_init_fence();
        for (int s = 0; s < BULK_DEPTH; s++)
            if (w0 + s * W < ntiles) issue(w0 + s * W, s);
    }
    __syncwarp();
    uint32_t i = 0;
    for (uint32_t tile = w0; tile < ntiles; tile += W, i++) {
        const int s = int(i % BULK_DEPTH);
        int ok = 1;
        if (lane == 0) ok = mbar_wait_bounded(smem_addr(&bars[warp][s]), (i / BULK_DEPTH) & 1) ? 1 : 0;
        ok = __shfl_sync(0xFFFFFFFFu, ok, 0);
        if (!ok) {
            if (lane == 0) bulk_abort(bars, warp, i, tile, W, ntiles, err);
            return;
        }
        const cplx<T> *b = buf + s * BULK_AMPS;
        cplx<T> v[BULK_PPL];
        uint32_t loc[BULK_PPL];
#pragma unroll
        for (int q = 0; q < BULK_PPL; q++) {
            const uint32_t p = lane + 32 * q;
            loc[q] = wide ? p : (ins0<uint32_t>(p, t) | bit);
            v[q] = b[loc[q]];
        }
        __syncwarp();
        if (lane == 0) {
            fence_proxy_async_smem();
            if (tile + BULK_DEPTH * W < ntiles) issue(tile + BULK_DEPTH * W, s);
        }
        const uint32_t a = first_amp(tile);
#pragma unroll
        for (int q = 0; q < BULK_PPL; q++) {
            diag_update<T, OP>(v[q], k, (pt >> (8 * (q % 3))) & 0xFFu);
            st[a + loc[q]] = v[q];
        }
    }
}

// collapse (measure.cpp:31-57): keep half scaled by `factor`, other half zero.
template <class T>
__global__ void __launch_bounds__(256) k_collapse(cplx<T> *__restrict__ st, uint64_t npairs,
                                                  unsigned t, unsigned outcome, T factor)
{
    const uint64_t bit = uint64_t(1) << t;
    const uint64_t keep = outcome ? bit : 0, drop = outcome ? 0 : bit;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < npairs; j += stride) {
        uint64_t i = insert0(j, t);
        cplx<T> a = st[i | keep];
        a.x = rn<T>::mul(a.x, factor);
        a.y = rn<T>::mul(a.y, factor);
        st[i | keep] = a;
        cplx<T> z;
        z.x = T(0);
        z.y = T(0);
        st[i | drop] = z;
    }
}

// complex64 amplitudes scaled in double and rounded once (precision form)
__global__ void __launch_bounds__(256) k_collapse_f64(float2 *__restrict__ st, uint64_t npairs,
                                                      unsigned t, unsigned outcome, double factor)
{
    const uint64_t bit = uint64_t(1) << t;
    const uint64_t keep = outcome ? bit : 0, drop = outcome ? 0 : bit;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < npairs; j += stride) {
        uint64_t i = insert0(j, t);
        float2 a = st[i | keep];
        a.x = float(double(a.x) * factor);
        a.y = float(double(a.y) * factor);
        st[i | keep] = a;
        st[i | drop] = make_float2(0.f, 0.f);
    }
}

template <class T>
__global__ void k_set_one(cplx<T> *st, uint64_t pos)
{
    cplx<T> one;
    one.x = T(1);
    one.y = T(0);
    st[pos] = one;
}

// The staged sweeps take complex128 states of up to 31 qubits (32-bit
// indices) with at least one whole tile, when QSLC_BULK=1.  They are not
// the default: on dense 28-qubit states the register sweeps run rotations
// at 5.56-5.67 TB/s and phase at 5.36-5.38, the best staged shape (8 warps,
// 2 buffers, 4 pairs per lane, 3 CTAs per SM) at 5.28-5.35 and 5.11.
inline bool bulk_enabled()
{
    static const bool on = [] {
        const char *e = std::getenv("QSLC_BULK");
        return e && e[0] == '1';
    }();
    return on;
}

// The warp-exchange sweeps (k_pair1_shfl) take one-qubit pair gates on
// targets 0-4 of states of at least 5 qubits.  By default only pauliX and
// pauliY, which move amplitudes without arithmetic: on a dense 28-qubit
// state they run at 6.64-6.67 TB/s there against 6.16-6.69 for the
// register sweeps.  The rotations and Hadamard stay on the register sweeps
// (5.43-5.82 TB/s against 4.89-5.30 exchanged), whose thread computes both
// outputs of a pair from operands it decodes once.  QSLC_SHFL=1 sends every
// pair gate on those targets through the exchange, QSLC_SHFL=0 none.
inline int shfl_mode()
{
    static const int m = [] {
        const char *e = std::getenv("QSLC_SHFL");
        return e && e[0] == '1' ? 1 : e && e[0] == '0' ? 0 : -1;
    }();
    return m;
}

inline bool use_shfl(int op, unsigned t, unsigned n)
{
    if (t >= 5 || n < 5) return false;
    const int m = shfl_mode();
    return m == 1 || (m == -1 && (op == P_SWAP || op == P_Y));
}

template <class T>
bool use_bulk(const qslc_state *s)
{
    return sizeof(T) == 8 && s->n >= unsigned(BULK_LOG2 + 1) && s->n <= 31 && bulk_enabled();
}

// Launch a staged sweep: a persistent grid of up to BULK_CTAS_PER_SM CTAs
// per SM, each with its warps' buffers in dynamic shared memory.
template <class T, class K>
int launch_bulk(qslc_state *s, K kernel, uint32_t ntiles, unsigned t, const Coef<T> &k, unsigned pat)
{
    int rc = ensure_wait_err(s);
    if (rc) return rc;
    // per kernel: its shared-memory limit raised once, and the CTAs of it
    // that fit on an SM, which sizes the persistent grid
    static std::vector<std::pair<const void *, int>> configured;
    const void *key = reinterpret_cast<const void *>(kernel);
    int per_sm = 0;
    for (const auto &c : configured)
        if (c.first == key) per_sm = c.second;
    if (!per_sm) {
        QSLC_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(bulk_smem_bytes<T>())));
        QSLC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, BULK_WARPS * 32,
                                                                bulk_smem_bytes<T>()));
        if (per_sm < 1) return fail(QSLC_ECUDA, "a staged sweep does not fit on an SM");
        if (per_sm > BULK_CTAS_PER_SM) per_sm = BULK_CTAS_PER_SM;
        configured.emplace_back(key, per_sm);
    }
    uint64_t blocks = (uint64_t(ntiles) + BULK_WARPS - 1) / BULK_WARPS;
    const uint64_t cap = uint64_t(sm_count()) * unsigned(per_sm);
    if (blocks > cap) blocks = cap;
    kernel<<<unsigned(blocks), BULK_WARPS * 32, bulk_smem_bytes<T>(), s->stream>>>(
        static_cast<cplx<T> *>(s->amps), ntiles, t, k, pat, s->wait_err);
    s->wait_err_pending = true;
    return QSLC_OK;
}

// Sweeps of states of up to 31 qubits index in 32 bits (fewer integer
// operations per amplitude); larger states in 64 bits.
template <class F>
void with_index(unsigned n, F &&f)
{
    if (n <= 31) f(uint32_t(0));
    else f(uint64_t(0));
}

template <class T>
int gate1_t(qslc_state *s, int gate, unsigned t, double angle)
{
    auto *st = static_cast<cplx<T> *>(s->amps);
    const uint64_t half = uint64_t(1) << (s->n - 1);
    const unsigned grid = grid_for(half);
    cudaStream_t str = s->stream;
    const bool dp = sizeof(T) == 8;
    const unsigned rot = dp ? pattern_rot() : 0, had = dp ? pattern_h() : 0, dg = dp ? pattern_diag() : 0;
    const bool bulk = use_bulk<T>(s);
    const uint32_t ntiles = bulk ? uint32_t(half / BULK_PAIRS) : 0;
    int brc = QSLC_OK;
    auto pair = [&](auto op, unsigned pat0, const Coef<T> &k, auto cands) {
        constexpr int OP = decltype(op)::value;
        const unsigned pat = OP == P_H ? pat0 : pattern_for(k, pat0);
        cands(pat, [&](auto c) {
            if (use_shfl(OP, t, s->n)) {
                with_index(s->n, [&](auto ix) {
                    k_pair1_shfl<T, OP, decltype(c)::value, decltype(ix)>
                        <<<grid_for(2 * half), 256, 0, str>>>(st, 2 * half, t, k, pat);
                });
                return;
            }
            if constexpr (sizeof(T) == 8) {
                if (bulk) {
                    brc = launch_bulk<T>(s, k_pair1_bulk<T, OP, decltype(c)::value>, ntiles, t, k, pat);
                    return;
                }
            }
            with_index(s->n, [&](auto ix) {
                k_pair1<T, OP, decltype(c)::value, decltype(ix)><<<grid, 256, 0, str>>>(st, half, t, k, pat);
            });
        });
    };
    auto rot_c = [](unsigned p, auto f) { with_pattern<QSLC_ROT_PATTERNS>(p, f); };
    auto h_c = [](unsigned p, auto f) { with_pattern<QSLC_H_PATTERNS>(p, f); };
    auto none = [](unsigned p, auto f) { with_pattern<0u>(p, f); };
    switch (gate) {
    case QSLC_PAULI_X: pair(std::integral_constant<int, P_SWAP>{}, 0, Coef<T>{}, none); break;
    case QSLC_PAULI_Y: pair(std::integral_constant<int, P_Y>{}, 0, Coef<T>{}, none); break;
    case QSLC_HADAMARD: pair(std::integral_constant<int, P_H>{}, had, sqrt2_coef<T>(), h_c); break;
    case QSLC_ROTATE_X: pair(std::integral_constant<int, P_RX>{}, rot, half_angle<T>(angle), rot_c); break;
    case QSLC_ROTATE_Y: pair(std::integral_constant<int, P_RY>{}, rot, half_angle<T>(angle), rot_c); break;
    case QSLC_ROTATE_Z: pair(std::integral_constant<int, P_RZ>{}, rot, half_angle<T>(angle), rot_c); break;
    case QSLC_PAULI_Z:
        if constexpr (sizeof(T) == 8) {
            if (bulk) {
                brc = launch_bulk<T>(s, k_diag1_bulk<T, D_NEG, 0u>, ntiles, t, Coef<T>{}, 0);
                break;
            }
        }
        with_index(s->n, [&](auto ix) {
            k_diag1<T, D_NEG, 0u, decltype(ix)><<<grid, 256, 0, str>>>(st, half, t, Coef<T>{}, 0);
        });
        break;
    case QSLC_PHASE: {
        const Coef<T> k = full_angle<T>(angle);
        const unsigned pd = pattern_for(k, dg);
        with_pattern<QSLC_DIAG_PATTERNS>(pd, [&](auto c) {
            if constexpr (sizeof(T) == 8) {
                if (bulk) {
                    brc = launch_bulk<T>(s, k_diag1_bulk<T, D_PHASE, decltype(c)::value>, ntiles, t, k, pd);
                    return;
                }
            }
            with_index(s->n, [&](auto ix) {
                k_diag1<T, D_PHASE, decltype(c)::value, decltype(ix)><<<grid, 256, 0, str>>>(st, half, t, k, pd);
            });
        });
        break;
    }
    default: return fail(QSLC_EINVAL, "unknown one-qubit gate code " + std::to_string(gate));
    }
    if (brc) return brc;
    s->launches++;
    QSLC_CUDA(cudaGetLastError());
    return QSLC_OK;
}

template <class T>
int gate2_t(qslc_state *s, int gate, unsigned q1, unsigned q2, double angle)
{
    auto *st = static_cast<cplx<T> *>(s->amps);
    const uint64_t quads = uint64_t(1) << (s->n - 2);
    const unsigned lo = q1 < q2 ? q1 : q2, hi = q1 < q2 ? q2 : q1;
    const uint64_t b1 = uint64_t(1) << q1, b2 = uint64_t(1) << q2;
    const unsigned grid = grid_for(quads);
    cudaStream_t str = s->stream;
    const bool dp = sizeof(T) == 8;
    const unsigned rot = dp ? pattern_rot() : 0, had = dp ? pattern_h() : 0, dg = dp ? pattern_diag() : 0;
    // pair kernel with operation OP, mode MODE, pattern pat among candidates
    auto pair = [&](auto op, auto mode, unsigned pat0, const Coef<T> &k, auto cands) {
        constexpr int OP = decltype(op)::value, MODE = decltype(mode)::value;
        const unsigned pat = OP == P_H ? pat0 : pattern_for(k, pat0);
        cands(pat, [&](auto c) {
            with_index(s->n, [&](auto ix) {
                k_pair2<T, OP, MODE, decltype(c)::value, decltype(ix)><<<grid, 256, 0, str>>>(st, quads, lo, hi, b1, b2,
                                                                                            k, pat);
            });
        });
    };
    auto rot_c = [](unsigned p, auto f) { with_pattern<QSLC_ROT2_PATTERNS>(p, f); };
    auto h_c = [](unsigned p, auto f) { with_pattern<QSLC_H_PATTERNS>(p, f); };
    auto none = [](unsigned p, auto f) { with_pattern<0u>(p, f); };
    using M0 = std::integral_constant<int, 0>;
    using M1 = std::integral_constant<int, 1>;
    using M2 = std::integral_constant<int, 2>;
    switch (gate) {
    case QSLC_CONTROL_NOT: pair(std::integral_constant<int, P_SWAP>{}, M0{}, 0, Coef<T>{}, none); break;
    case QSLC_CONTROL_Y: pair(std::integral_constant<int, P_Y>{}, M0{}, 0, Coef<T>{}, none); break;
    case QSLC_CONTROL_ROTATE_X:
        pair(std::integral_constant<int, P_RX>{}, M0{}, rot, half_angle<T>(angle), rot_c);
        break;
    case QSLC_CONTROL_ROTATE_Y:
        pair(std::integral_constant<int, P_RY>{}, M0{}, rot, half_angle<T>(angle), rot_c);
        break;
    case QSLC_CONTROL_ROTATE_Z:
        pair(std::integral_constant<int, P_RZ>{}, M0{}, rot, half_angle<T>(angle), rot_c);
        break;
    case QSLC_CONTROL_HADAMARD: pair(std::integral_constant<int, P_H>{}, M0{}, had, sqrt2_coef<T>(), h_c); break;
    case QSLC_SWAP: pair(std::integral_constant<int, P_SWAP>{}, M1{}, 0, Coef<T>{}, none); break;
    case QSLC_NP_ROTATE_X:
        pair(std::integral_constant<int, P_RX>{}, M1{}, rot, half_angle<T>(angle), rot_c);
        break;
    case QSLC_NP_ROTATE_Y:
        pair(std::integral_constant<int, P_RY>{}, M1{}, rot, half_angle<T>(angle), rot_c);
        break;
    case QSLC_NP_HADAMARD: pair(std::integral_constant<int, P_H>{}, M1{}, had, sqrt2_coef<T>(), h_c); break;
    case QSLC_FSWAP: pair(std::integral_constant<int, P_SWAP>{}, M2{}, 0, Coef<T>{}, none); break;
    case QSLC_CONTROL_Z:
        with_index(s->n, [&](auto ix) {
            k_diag2<T, D_NEG, 0u, decltype(ix)><<<grid, 256, 0, str>>>(st, quads, lo, hi, b1 | b2, Coef<T>{}, 0);
        });
        break;
    case QSLC_CONTROL_PHASE: {
        const Coef<T> k = full_angle<T>(angle);
        const unsigned pd = pattern_for(k, dg);
        with_pattern<QSLC_DIAG_PATTERNS>(pd, [&](auto c) {
            with_index(s->n, [&](auto ix) {
                k_diag2<T, D_PHASE, decltype(c)::value, decltype(ix)><<<grid, 256, 0, str>>>(st, quads, lo, hi, b1 | b2,
                                                                                         k, pd);
            });
        });
        break;
    }
    default: return fail(QSLC_EINVAL, "unknown two-qubit gate code " + std::to_string(gate));
    }
    s->launches++;
    QSLC_CUDA(cudaGetLastError());
    return QSLC_OK;
}

// A plain one-qubit gate as a group member: its op and coefficients.
template <class T>
void group_member(const GateOp &g, int &op, Coef<T> &k)
{
    k = Coef<T>{};
    switch (g.code) {
    case QSLC_PAULI_X: op = P_SWAP; break;
    case QSLC_PAULI_Y: op = P_Y; break;
    case QSLC_PAULI_Z: op = GROUP_DIAG + D_NEG; break;
    case QSLC_HADAMARD: op = P_H; k = sqrt2_coef<T>(); break;
    case QSLC_PHASE: op = GROUP_DIAG + D_PHASE; k = full_angle<T>(g.angle); break;
    case QSLC_ROTATE_X: op = P_RX; k = half_angle<T>(g.angle); break;
    case QSLC_ROTATE_Y: op = P_RY; k = half_angle<T>(g.angle); break;
    default: op = P_RZ; k = half_angle<T>(g.angle); break;
    }
}

template <class T>
int group2_t(qslc_state *s, const GateOp &g0, const GateOp &g1)
{
    GroupGates<T> g;
    group_member<T>(g0, g.op[0], g.k[0]);
    group_member<T>(g1, g.op[1], g.k[1]);
    const unsigned lo = g0.q1 < g1.q1 ? g0.q1 : g1.q1, hi = g0.q1 < g1.q1 ? g1.q1 : g0.q1;
    const uint64_t quads = uint64_t(1) << (s->n - 2);
    auto *st = static_cast<cplx<T> *>(s->amps);
    with_index(s->n, [&](auto ix) {
        using IX = decltype(ix);
        k_group2<T, IX><<<grid_for(quads), 256, 0, s->stream>>>(st, quads, lo, hi, IX(1) << g0.q1,
                                                               IX(1) << g1.q1, g);
    });
    s->launches++;
    QSLC_CUDA(cudaGetLastError());
    return QSLC_OK;
}

}  // namespace

// Grouping is on unless QSLC_GROUP=0.
bool grouping_enabled()
{
    static const bool on = [] {
        const char *e = std::getenv("QSLC_GROUP");
        return !(e && e[0] == '0');
    }();
    return on;
}

int launch_group2(qslc_state *s, const GateOp &g0, const GateOp &g1)
{
    return s->dtype == QSLC_C128 ? group2_t<double>(s, g0, g1) : group2_t<float>(s, g0, g1);
}

int debug_bounds_error()
{
#ifdef QSLC_DEBUG_BOUNDS
    unsigned long long bad = 0;
    QSLC_CUDA(cudaDeviceSynchronize());
    QSLC_CUDA(cudaMemcpyFromSymbol(&bad, g_bad_index, sizeof(bad)));
    if (bad) {
        const unsigned long long zero = 0;
        QSLC_CUDA(cudaMemcpyToSymbol(g_bad_index, &zero, sizeof(zero)));
        return fail(QSLC_EINVAL, "a sweep indexed outside the state (debug bounds check): index " +
                                     std::to_string(bad - 1));
    }
#endif
    return QSLC_OK;
}

int launch_gate1(qslc_state *s, int gate, unsigned targ, double angle)
{
    return s->dtype == QSLC_C128 ? gate1_t<double>(s, gate, targ, angle)
                                 : gate1_t<float>(s, gate, targ, angle);
}

int launch_gate2(qslc_state *s, int gate, unsigned q1, unsigned q2, double angle)
{
    return s->dtype == QSLC_C128 ? gate2_t<double>(s, gate, q1, q2, angle)
                                 : gate2_t<float>(s, gate, q1, q2, angle);
}

int launch_collapse(qslc_state *s, unsigned targ, unsigned outcome, double factor)
{
    const uint64_t half = uint64_t(1) << (s->n - 1);
    const unsigned grid = grid_for(half);
    if (s->dtype == QSLC_C128)
        k_collapse<double><<<grid, 256, 0, s->stream>>>(static_cast<double2 *>(s->amps), half, targ,
                                                        outcome, factor);
    else
        k_collapse<float><<<grid, 256, 0, s->stream>>>(static_cast<float2 *>(s->amps), half, targ,
                                                       outcome, float(factor));
    s->launches++;
    QSLC_CUDA(cudaGetLastError());
    return QSLC_OK;
}

int launch_collapse_f64(qslc_state *s, unsigned targ, unsigned outcome, double factor)
{
    const uint64_t half = uint64_t(1) << (s->n - 1);
    k_collapse_f64<<<grid_for(half), 256, 0, s->stream>>>(static_cast<float2 *>(s->amps), half, targ,
                                                        outcome, factor);
    s->launches++;
    QSLC_CUDA(cudaGetLastError());
    return QSLC_OK;
}

// All amplitudes zero except `pos`, which becomes 1 (default.cpp:57-65, :80-90).
int launch_fill_basis(qslc_state *s, uint64_t pos)
{
    if (!s->amps || pos >= s->namps)
        return fail(QSLC_EINVAL, "basis position " + std::to_string(pos) + " outside the " +
                                     std::to_string(s->namps) + " stored amplitudes");
    QSLC_CUDA(cudaMemsetAsync(s->amps, 0, s->namps * s->amp_bytes(), s->stream));
    if (s->dtype == QSLC_C128)
        k_set_one<double><<<1, 1, 0, s->stream>>>(static_cast<double2 *>(s->amps), pos);
    else
        k_set_one<float><<<1, 1, 0, s->stream>>>(static_cast<float2 *>(s->amps), pos);
    s->launches++;
    QSLC_CUDA(cudaGetLastError());
    return QSLC_OK;
}

}  // namespace qslc
