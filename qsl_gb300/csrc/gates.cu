// gates.cu -- amplitude-pair sweeps of the plain (2^n) layout.
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
#include "dpemu.cuh"

#include <cmath>
#include <cstdlib>

namespace qslc {
namespace {

enum PairOp { P_SWAP, P_Y, P_H, P_RX, P_RY, P_RZ };
enum DiagOp { D_NEG, D_PHASE };

template <class T>
struct Coef {
    T c, s;  // cos/sin of angle/2 (rotations) or of angle (phase); sqrt2 for H
    emu::MulConst kc, ks;   // c and s decoded for the integer path (double only)
    emu::DivConst kd;       // c as a divisor (Hadamard)
};

// One Hadamard output, RN(RN(a +- b) / sqrt2) (gates.cpp:95-98).  The
// division always runs on the integer pipes (an FP64 divide is a long
// iteration on the FP64 pipe); with EMU the sum does too.
template <class T, bool EMU, bool NEG>
__device__ __forceinline__ T hdiv(T a, T b, const Coef<T> &k)
{
    using R = rn<T>;
    if constexpr (sizeof(T) == 8) {
        bool ok = k.kd.usable != 0;
        if (ok) {
            uint64_t sb;
            if constexpr (EMU) sb = emu::add_rn(emu::dbits(a), emu::dbits(b) ^ (NEG ? emu::SIGN : 0), ok);
            else sb = emu::dbits(NEG ? R::sub(a, b) : R::add(a, b));
            const uint64_t q = emu::div_rn(sb, k.kd, ok);
            if (ok) return emu::dfrom(q);
        }
    }
    return R::div(NEG ? R::sub(a, b) : R::add(a, b), k.c);
}

// One output of a rotation or phase update: RN(RN(a*k1) + RN(b*k2)), or
// RN(RN(a*k1) - RN(b*k2)) when NEG.  With EMU the integer pipes compute it
// (dpemu.cuh), falling back to the FP64 pipe for operands the integer path
// declines; either way the bits are the reference's.
template <class T, bool EMU, bool NEG>
__device__ __forceinline__ T dot2(T a, T k1, const emu::MulConst &e1, T b, T k2,
                                  const emu::MulConst &e2)
{
    if constexpr (EMU && sizeof(T) == 8) {
        bool ok = (e1.usable & e2.usable) != 0;
        if (ok) {
            const uint64_t r = emu::dot2_rn(emu::dbits(a), e1, emu::dbits(b), e2, NEG, ok);
            if (ok) return emu::dfrom(r);
        }
    }
    using R = rn<T>;
    return NEG ? R::sub(R::mul(a, k1), R::mul(b, k2)) : R::add(R::mul(a, k1), R::mul(b, k2));
}

// EM: bit i set = output i (r0.x, r0.y, r1.x, r1.y) on the integer pipes.
template <class T, int OP, int EM = 0>
__device__ __forceinline__ void pair_update(cplx<T> &a0, cplx<T> &a1, const Coef<T> &k)
{
    using R = rn<T>;
    cplx<T> r0, r1;
    constexpr bool E0 = EM & 1, E1 = EM & 2, E2 = EM & 4, E3 = EM & 8;
    if constexpr (OP == P_SWAP) {            // gates.cpp:41, :236, :524
        r0 = a1;
        r1 = a0;
    } else if constexpr (OP == P_Y) {        // gates.cpp:59-62, :267-270
        r0.x = a1.y; r0.y = -a1.x;
        r1.x = -a0.y; r1.y = a0.x;
    } else if constexpr (OP == P_H) {        // gates.cpp:95-98, :493-496, :675-678
        r0.x = hdiv<T, E0, false>(a0.x, a1.x, k);
        r0.y = hdiv<T, E1, false>(a0.y, a1.y, k);
        r1.x = hdiv<T, E2, true>(a0.x, a1.x, k);
        r1.y = hdiv<T, E3, true>(a0.y, a1.y, k);
    } else if constexpr (OP == P_RX) {       // gates.cpp:139-144, :336-341, :595-600
        r0.x = dot2<T, E0, false>(a0.x, k.c, k.kc, a1.y, k.s, k.ks);
        r0.y = dot2<T, E1, true>(a0.y, k.c, k.kc, a1.x, k.s, k.ks);
        r1.x = dot2<T, E2, false>(a1.x, k.c, k.kc, a0.y, k.s, k.ks);
        r1.y = dot2<T, E3, true>(a1.y, k.c, k.kc, a0.x, k.s, k.ks);
    } else if constexpr (OP == P_RY) {       // gates.cpp:169-174, :380-385, :638-643
        r0.x = dot2<T, E0, true>(a0.x, k.c, k.kc, a1.x, k.s, k.ks);
        r0.y = dot2<T, E1, true>(a0.y, k.c, k.kc, a1.y, k.s, k.ks);
        r1.x = dot2<T, E2, false>(a0.x, k.s, k.ks, a1.x, k.c, k.kc);
        r1.y = dot2<T, E3, false>(a0.y, k.s, k.ks, a1.y, k.c, k.kc);
    } else {                                 // P_RZ: gates.cpp:200-205, :424-429
        r0.x = dot2<T, E0, false>(a0.x, k.c, k.kc, a0.y, k.s, k.ks);
        r0.y = dot2<T, E1, true>(a0.y, k.c, k.kc, a0.x, k.s, k.ks);
        r1.x = dot2<T, E2, true>(a1.x, k.c, k.kc, a1.y, k.s, k.ks);
        r1.y = dot2<T, E3, false>(a1.y, k.c, k.kc, a1.x, k.s, k.ks);
    }
    a0 = r0;
    a1 = r1;
}

template <class T, int OP, int EM = 0>
__device__ __forceinline__ void diag_update(cplx<T> &a, const Coef<T> &k)
{
    using R = rn<T>;
    if constexpr (OP == D_NEG) {             // gates.cpp:76-77, :296-297 (x *= -1)
        a.x = R::mul(a.x, T(-1));
        a.y = R::mul(a.y, T(-1));
    } else {                                 // gates.cpp:114-115, :460-461
        T x = a.x, y = a.y;
        a.x = dot2<T, (EM & 1) != 0, true>(x, k.c, k.kc, y, k.s, k.ks);
        a.y = dot2<T, (EM & 2) != 0, false>(y, k.c, k.kc, x, k.s, k.ks);
    }
}

// One-qubit pair gates: pairs (i0, i0 + 2^t), i0 = insert0(j, t).
template <class T, int OP, int EM = 0>
__global__ void __launch_bounds__(256) k_pair1(cplx<T> *__restrict__ st, uint64_t npairs,
                                               unsigned t, Coef<T> k)
{
    const uint64_t bit = uint64_t(1) << t;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < npairs; j += stride) {
        uint64_t i0 = insert0(j, t);
        cplx<T> a0 = st[i0], a1 = st[i0 | bit];
        pair_update<T, OP, EM>(a0, a1, k);
        st[i0] = a0;
        st[i0 | bit] = a1;
    }
}

// One-qubit diagonal gates on the |1> half: index insert0(j, t) | 2^t.
template <class T, int OP, int EM = 0>
__global__ void __launch_bounds__(256) k_diag1(cplx<T> *__restrict__ st, uint64_t count,
                                               unsigned t, Coef<T> k)
{
    const uint64_t bit = uint64_t(1) << t;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < count; j += stride) {
        uint64_t i = insert0(j, t) | bit;
        cplx<T> a = st[i];
        diag_update<T, OP, EM>(a, k);
        st[i] = a;
    }
}

// rotateZ touches both halves with different coefficients; it is a pair
// gate whose two members do not mix (gates.cpp:181-209).

// Two-qubit gates: j in [0, 2^(n-2)), base = j with zeros inserted at lo < hi.
// MODE 0: controlled pair (base|b1, base|b1|b2), b1 = control bit;
// MODE 1: number-preserving pair (base|b1, base|b2);
// MODE 2: fswap = MODE 1 swap plus negation of base|b1|b2.
template <class T, int OP, int MODE, int EM = 0>
__global__ void __launch_bounds__(256) k_pair2(cplx<T> *__restrict__ st, uint64_t nquads,
                                               unsigned lo, unsigned hi, uint64_t b1,
                                               uint64_t b2, Coef<T> k)
{
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < nquads; j += stride) {
        uint64_t base = insert00(j, lo, hi);
        uint64_t x1 = base | b1;
        uint64_t x2 = (MODE == 0) ? (x1 | b2) : (base | b2);
        cplx<T> a0 = st[x1], a1 = st[x2];
        pair_update<T, OP, EM>(a0, a1, k);
        st[x1] = a0;
        st[x2] = a1;
        if constexpr (MODE == 2) {
            uint64_t x3 = base | b1 | b2;
            cplx<T> a = st[x3];
            diag_update<T, D_NEG>(a, k);
            st[x3] = a;
        }
    }
}

// controlZ / controlPhase: the |11> quarter (gates.cpp:277-301, :436-465).
template <class T, int OP, int EM = 0>
__global__ void __launch_bounds__(256) k_diag2(cplx<T> *__restrict__ st, uint64_t nquads,
                                               unsigned lo, unsigned hi, uint64_t both,
                                               Coef<T> k)
{
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < nquads; j += stride) {
        uint64_t i = insert00(j, lo, hi) | both;
        cplx<T> a = st[i];
        diag_update<T, OP, EM>(a, k);
        st[i] = a;
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

// Host-side coefficients, computed exactly as the reference does: in Fp,
// with std::cos/std::sin of angle/2 (gates.cpp:124-125) or of angle
// (:106), and sqrt2 = Fp(std::sqrt(2)) (:94).
template <class T>
Coef<T> coef(T c, T s)
{
    Coef<T> k{};
    k.c = c;
    k.s = s;
    k.kc = emu::make_const(double(c));
    k.ks = emu::make_const(double(s));
    k.kd = emu::make_div(double(c));
    return k;
}
template <class T>
Coef<T> half_angle(double angle)
{
    T a = T(angle);
    return coef<T>(T(std::cos(a / 2)), T(std::sin(a / 2)));
}
template <class T>
Coef<T> full_angle(double angle)
{
    T a = T(angle);
    return coef<T>(T(std::cos(a)), T(std::sin(a)));
}
template <class T>
Coef<T> sqrt2_coef()
{
    return coef<T>(T(std::sqrt(2)), T(0));
}

// Share of the dense updates' outputs computed on the integer pipes
// (a mask over the four outputs of a pair, two of a diagonal update).
// QSLC_EMU_MASK overrides it for tuning sweeps.
int emu_mask_pair()
{
    static int m = [] {
        const char *e = std::getenv("QSLC_EMU_MASK");
        return e ? std::atoi(e) & 15 : 5;
    }();
    return m;
}
int emu_mask_diag()
{
    static int m = [] {
        const char *e = std::getenv("QSLC_EMU_MASK_DIAG");
        return e ? std::atoi(e) & 3 : 1;
    }();
    return m;
}

// launch a kernel template instantiated for the current emulation mask
#define WITH_PAIR_MASK(T, CALL)                                      \
    do {                                                             \
        if constexpr (sizeof(T) == 8) {                              \
            switch (emu_mask_pair()) {                               \
            case 1: { constexpr int EMV = 1; CALL; } break;          \
            case 3: { constexpr int EMV = 3; CALL; } break;          \
            case 7: { constexpr int EMV = 7; CALL; } break;          \
            case 15: { constexpr int EMV = 15; CALL; } break;        \
            case 5: { constexpr int EMV = 5; CALL; } break;          \
            default: { constexpr int EMV = 0; CALL; } break;         \
            }                                                        \
        } else {                                                     \
            constexpr int EMV = 0;                                   \
            CALL;                                                    \
        }                                                            \
    } while (0)
#define WITH_DIAG_MASK(T, CALL)                                      \
    do {                                                             \
        if constexpr (sizeof(T) == 8) {                              \
            switch (emu_mask_diag()) {                               \
            case 1: { constexpr int EMV = 1; CALL; } break;          \
            case 2: { constexpr int EMV = 2; CALL; } break;          \
            case 3: { constexpr int EMV = 3; CALL; } break;          \
            default: { constexpr int EMV = 0; CALL; } break;         \
            }                                                        \
        } else {                                                     \
            constexpr int EMV = 0;                                   \
            CALL;                                                    \
        }                                                            \
    } while (0)

template <class T>
int gate1_t(qslc_state *s, int gate, unsigned t, double angle)
{
    auto *st = static_cast<cplx<T> *>(s->amps);
    const uint64_t half = uint64_t(1) << (s->n - 1);
    const unsigned grid = grid_for(half);
    cudaStream_t str = s->stream;
    switch (gate) {
    case QSLC_PAULI_X: k_pair1<T, P_SWAP><<<grid, 256, 0, str>>>(st, half, t, Coef<T>{}); break;
    case QSLC_PAULI_Y: k_pair1<T, P_Y><<<grid, 256, 0, str>>>(st, half, t, Coef<T>{}); break;
    case QSLC_HADAMARD:
        WITH_PAIR_MASK(T, (k_pair1<T, P_H, EMV><<<grid, 256, 0, str>>>(st, half, t, sqrt2_coef<T>())));
        break;
    case QSLC_ROTATE_X:
        WITH_PAIR_MASK(T, (k_pair1<T, P_RX, EMV><<<grid, 256, 0, str>>>(st, half, t, half_angle<T>(angle))));
        break;
    case QSLC_ROTATE_Y:
        WITH_PAIR_MASK(T, (k_pair1<T, P_RY, EMV><<<grid, 256, 0, str>>>(st, half, t, half_angle<T>(angle))));
        break;
    case QSLC_ROTATE_Z:
        WITH_PAIR_MASK(T, (k_pair1<T, P_RZ, EMV><<<grid, 256, 0, str>>>(st, half, t, half_angle<T>(angle))));
        break;
    case QSLC_PAULI_Z: k_diag1<T, D_NEG><<<grid, 256, 0, str>>>(st, half, t, Coef<T>{}); break;
    case QSLC_PHASE:
        WITH_DIAG_MASK(T, (k_diag1<T, D_PHASE, EMV><<<grid, 256, 0, str>>>(st, half, t, full_angle<T>(angle))));
        break;
    default: return fail(QSLC_EINVAL, "unknown one-qubit gate code " + std::to_string(gate));
    }
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
#define P2(OP, MODE, K) k_pair2<T, OP, MODE><<<grid, 256, 0, str>>>(st, quads, lo, hi, b1, b2, K)
#define P2E(OP, MODE, K) \
    WITH_PAIR_MASK(T, (k_pair2<T, OP, MODE, EMV><<<grid, 256, 0, str>>>(st, quads, lo, hi, b1, b2, K)))
    switch (gate) {
    case QSLC_CONTROL_NOT: P2(P_SWAP, 0, Coef<T>{}); break;
    case QSLC_CONTROL_Y: P2(P_Y, 0, Coef<T>{}); break;
    case QSLC_CONTROL_ROTATE_X: P2E(P_RX, 0, half_angle<T>(angle)); break;
    case QSLC_CONTROL_ROTATE_Y: P2E(P_RY, 0, half_angle<T>(angle)); break;
    case QSLC_CONTROL_ROTATE_Z: P2E(P_RZ, 0, half_angle<T>(angle)); break;
    case QSLC_CONTROL_HADAMARD: P2E(P_H, 0, sqrt2_coef<T>()); break;
    case QSLC_SWAP: P2(P_SWAP, 1, Coef<T>{}); break;
    case QSLC_NP_ROTATE_X: P2E(P_RX, 1, half_angle<T>(angle)); break;
    case QSLC_NP_ROTATE_Y: P2E(P_RY, 1, half_angle<T>(angle)); break;
    case QSLC_NP_HADAMARD: P2E(P_H, 1, sqrt2_coef<T>()); break;
    case QSLC_FSWAP: P2(P_SWAP, 2, Coef<T>{}); break;
    case QSLC_CONTROL_Z:
        k_diag2<T, D_NEG><<<grid, 256, 0, str>>>(st, quads, lo, hi, b1 | b2, Coef<T>{});
        break;
    case QSLC_CONTROL_PHASE:
        WITH_DIAG_MASK(T, (k_diag2<T, D_PHASE, EMV><<<grid, 256, 0, str>>>(st, quads, lo, hi, b1 | b2,
                                                                            full_angle<T>(angle))));
        break;
    default: return fail(QSLC_EINVAL, "unknown two-qubit gate code " + std::to_string(gate));
    }
#undef P2
#undef P2E
    s->launches++;
    QSLC_CUDA(cudaGetLastError());
    return QSLC_OK;
}

}  // namespace

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
