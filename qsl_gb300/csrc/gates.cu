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
#include "gatemath.cuh"

#include <cmath>
#include <cstdlib>

namespace qslc {
namespace {


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
            if (j + r * stride < npairs) {
                a0[r] = st[i0[r]];
                a1[r] = st[i0[r] | bit];
            }
        }
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            if (j + r * stride < npairs) {
                pair_update<T, OP>(a0[r], a1[r], k, (pt >> (8 * r)) & 0xFFu);
                st[i0[r]] = a0[r];
                st[i0[r] | bit] = a1[r];
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
            if (j + r * stride < count) a[r] = st[i[r]];
        }
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            if (j + r * stride < count) {
                diag_update<T, OP>(a[r], k, (pt >> (8 * r)) & 0xFFu);
                st[i[r]] = a[r];
            }
        }
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
            if (j + r * stride < nquads) {
                a0[r] = st[x1[r]];
                a1[r] = st[x2[r]];
            }
        }
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            if (j + r * stride < nquads) {
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
            if (j + r * stride < nquads) a[r] = st[i[r]];
        }
#pragma unroll
        for (int r = 0; r < ITEMS; r++) {
            if (j + r * stride < nquads) {
                diag_update<T, OP>(a[r], k, (pt >> (8 * r)) & 0xFFu);
                st[i[r]] = a[r];
            }
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
    auto pair = [&](auto op, unsigned pat0, const Coef<T> &k, auto cands) {
        constexpr int OP = decltype(op)::value;
        const unsigned pat = OP == P_H ? pat0 : pattern_for(k, pat0);
        cands(pat, [&](auto c) {
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
        with_index(s->n, [&](auto ix) {
            k_diag1<T, D_NEG, 0u, decltype(ix)><<<grid, 256, 0, str>>>(st, half, t, Coef<T>{}, 0);
        });
        break;
    case QSLC_PHASE: {
        const Coef<T> k = full_angle<T>(angle);
        const unsigned pd = pattern_for(k, dg);
        with_pattern<QSLC_DIAG_PATTERNS>(pd, [&](auto c) {
            with_index(s->n, [&](auto ix) {
                k_diag1<T, D_PHASE, decltype(c)::value, decltype(ix)><<<grid, 256, 0, str>>>(st, half, t, k, pd);
            });
        });
        break;
    }
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
