// replay.cuh -- exact replay of qsl's sequential floating-point sums.
//
// qsl computes prob() and the sampling CDF with a running sum in index
// order, s <- RN(s + p_i) (src/qubits/default/measure.cpp:60-78, :126-147).
// A parallel reduction rounds differently, which moves measurement outcomes
// and, at 2^30 amplitudes, about one shot in a thousand to a neighbouring
// basis state.  This header holds the pieces that reproduce the sequential
// sum exactly while the amplitudes are read in parallel:
//
//   While the running sum stays inside one binade [2^e, 2^(e+1)) it lives on
//   the grid of step u_e = ulp(2^e), and each rounded add moves it by
//   u_e * rne(p / u_e) grid steps, an integer that does not depend on s
//   (except for exact ties, which depend on the parity of s / u_e).  A tile
//   of consecutive terms therefore advances the sum by u_e * D with
//   D = sum of those integers, as long as the sum neither starts outside
//   binade e nor reaches 2^(e+1) inside the tile and no tie occurs.  Tiles
//   that break one of these conditions (a handful per sum: the ones where
//   the running sum crosses a power of two) are replayed term by term.
//
// Everything here is __host__ __device__ so the same code runs in the
// kernels and in the host sequencer.
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define QSLC_HD __host__ __device__ __forceinline__
#else
#define QSLC_HD inline
#endif

namespace qslc {

template <class A> struct fp_traits;
template <> struct fp_traits<double> {
    using bits_t = uint64_t;
    static constexpr int MANT = 52;       // stored mantissa bits
    static constexpr int BIAS = 1023;
    static constexpr int EMIN = -1022;    // smallest normal binade
    static constexpr int EXPMASK = 0x7FF;
};
template <> struct fp_traits<float> {
    using bits_t = uint32_t;
    static constexpr int MANT = 23;
    static constexpr int BIAS = 127;
    static constexpr int EMIN = -126;
    static constexpr int EXPMASK = 0xFF;
};

template <class A>
QSLC_HD typename fp_traits<A>::bits_t to_bits(A x)
{
    typename fp_traits<A>::bits_t b;
#ifdef __CUDA_ARCH__
    if constexpr (sizeof(A) == 8) b = (uint64_t)__double_as_longlong(x);
    else b = (uint32_t)__float_as_uint(x);
#else
    std::memcpy(&b, &x, sizeof(A));
#endif
    return b;
}

// Binade of a positive normal x: the e with 2^e <= x < 2^(e+1).  Returns
// EMIN - 1 for zero and subnormals (no binade the fast path can use).
template <class A>
QSLC_HD int binade(A x)
{
    using T = fp_traits<A>;
    auto b = to_bits(x);
    int ef = int((b >> T::MANT) & T::EXPMASK);
    if (ef == 0) return T::EMIN - 1;
    return ef - T::BIAS;
}

// Integer number of grid steps of binade e that adding p >= 0 moves a sum
// of type A lying in binade e: rne(p / u_e) with u_e = 2^(e - MANT of A).
// `tie` is set when p / u_e is exactly half-way between two integers (the
// result then depends on the parity of the sum).  `big` is set when the
// step count does not fit the binade (p itself reaches 2^(e+1)).  The term
// may be of another type P (a float term held as a double, say): its value
// is decoded from its own format.
template <class A, class P = A>
QSLC_HD uint64_t grid_steps(P p, int e, bool &tie, bool &big)
{
    using T = fp_traits<A>;
    using TP = fp_traits<P>;
    tie = false;
    big = false;
    auto b = to_bits(p);
    int ef = int((b >> TP::MANT) & TP::EXPMASK);
    uint64_t m = uint64_t(b & ((typename TP::bits_t(1) << TP::MANT) - 1));
    if (ef == 0 && m == 0) return 0;
    int lsb;                                  // exponent of m's last bit
    if (ef != 0) {
        m |= uint64_t(1) << TP::MANT;
        lsb = ef - TP::BIAS - TP::MANT;
    } else {
        lsb = TP::EMIN - TP::MANT;
    }
    int sh = (e - T::MANT) - lsb;             // p / u_e = m * 2^-sh
    if (sh <= 0) {
        // exact multiple of the grid; 2^(MANT+1) steps or more leave the binade
        int ls = -sh;
        if (ls > T::MANT + 1 || (m >> (T::MANT + 1 - ls)) != 0) { big = true; return 0; }
        return m << ls;
    }
    // a term of more precision than the sum: its step count may not fit
    if (T::MANT + 1 + sh < 64 && (m >> (T::MANT + 1 + sh)) != 0) { big = true; return 0; }
    if (sh >= 64) return 0;                   // m < 2^53 <= half a step
    uint64_t q = m >> sh;
    uint64_t rem = m & ((uint64_t(1) << sh) - 1);
    uint64_t half = uint64_t(1) << (sh - 1);
    if (rem == half) tie = true;
    return q + (rem > half ? 1 : 0);
}

// The effect of a run of terms on a sum in binade e, as grid steps, for
// either parity of the sum (in grid steps) before the run.  A term whose
// quotient p / u_e sits exactly half-way (a tie) rounds to the even
// neighbour, so its step count is q or q + 1 depending on the parity of the
// sum it lands on; every other term has a fixed count.  Runs compose
// associatively: (A then B)(par) = A(par) + B(par + A(par)).
struct Tx {
    uint64_t d[2];
};
QSLC_HD Tx tx_identity() { return Tx{{0, 0}}; }
QSLC_HD Tx tx_term(uint64_t q, bool tie)
{
    if (!tie) return Tx{{q, q}};
    return Tx{{q + (q & 1), q + ((q + 1) & 1)}};
}
// Counts saturate at 2^62: a tile whose count reaches the binade's size
// is discarded anyway, and saturation keeps such a count from wrapping
// around to a small value.
constexpr uint64_t TX_SAT = uint64_t(1) << 62;
QSLC_HD uint64_t sat_add(uint64_t a, uint64_t b)
{
    const uint64_t r = a + b;   // a, b <= 2^62: no wrap
    return r > TX_SAT ? TX_SAT : r;
}
QSLC_HD Tx tx_then(const Tx &a, const Tx &b)
{
    Tx r;
    r.d[0] = sat_add(a.d[0], b.d[(a.d[0]) & 1]);
    r.d[1] = sat_add(a.d[1], b.d[(1 + a.d[1]) & 1]);
    return r;
}

// ceil(u / u_e) with u_e = 2^(e - MANT): the first grid position of binade
// e at or above u >= 0, saturating at TX_SAT.  A sum at grid position N of
// binade e has reached u exactly when grid_ceil(u, e) <= N.
template <class A>
QSLC_HD uint64_t grid_ceil(A u, int e)
{
    using T = fp_traits<A>;
    auto b = to_bits(u);
    int ef = int((b >> T::MANT) & T::EXPMASK);
    uint64_t m = uint64_t(b & ((typename T::bits_t(1) << T::MANT) - 1));
    if (ef == 0 && m == 0) return 0;
    int lsb;
    if (ef != 0) {
        m |= uint64_t(1) << T::MANT;
        lsb = ef - T::BIAS - T::MANT;
    } else {
        lsb = T::EMIN - T::MANT;
    }
    const int sh = (e - T::MANT) - lsb;       // u / u_e = m * 2^-sh
    if (sh <= 0) {
        const int ls = -sh;
        if (ls >= 62 - T::MANT) return TX_SAT; // m < 2^(MANT+1): m << ls < 2^62 below this
        return m << ls;
    }
    if (sh >= 64) return 1;                    // 0 < u / u_e < 1
    const uint64_t q = m >> sh;
    return q + ((m & ((uint64_t(1) << sh) - 1)) != 0 ? 1 : 0);
}

// Runs of consecutive terms of a running sum of type A in binade e, for
// walking a sequential sum a warp at a time: each lane takes one run (its
// terms get(0), get(1), ...), run_effect gives the run's Tx (composed across
// lanes by a scan), run_walk advances a grid position through the run from
// where the lanes before left it, and run_find locates the term at which
// the position reaches a target.  The position must stay below 2^(MANT+1)
// (the binade's end); run_walk stops before the first term that would take
// it there, or whose step count does not fit the binade.
template <class A, class Get>
QSLC_HD Tx run_effect(Get get, unsigned len, int e, bool &big_any)
{
    Tx t = tx_identity();
    for (unsigned r = 0; r < len; r++) {
        bool tie, big;
        const uint64_t q = grid_steps<A>(get(r), e, tie, big);
        big_any |= big;
        t = tx_then(t, tx_term(q, tie));
    }
    return t;
}

template <class A, class Get>
QSLC_HD unsigned run_walk(Get get, unsigned len, int e, uint64_t &pos)
{
    const uint64_t lim = uint64_t(1) << (fp_traits<A>::MANT + 1);
    for (unsigned r = 0; r < len; r++) {
        bool tie, big;
        const uint64_t q = grid_steps<A>(get(r), e, tie, big);
        if (big || pos >= lim) return r;
        const uint64_t step = tx_term(q, tie).d[pos & 1];
        if (step >= lim - pos) return r;
        pos += step;
    }
    return len;
}

template <class A, class Get>
QSLC_HD unsigned run_find(Get get, unsigned len, int e, uint64_t pos, uint64_t target)
{
    for (unsigned r = 0; r < len; r++) {
        bool tie, big;
        const uint64_t q = grid_steps<A>(get(r), e, tie, big);
        pos += tx_term(q, tie).d[pos & 1];
        if (pos >= target) return r;
    }
    return len;
}

// The value of type A at grid position `pos` of binade e (pos in
// [2^MANT, 2^(MANT+1))).
template <class A>
QSLC_HD A grid_at(uint64_t pos, int e)
{
    using T = fp_traits<A>;
    const auto b = typename T::bits_t((uint64_t(e + T::BIAS) << T::MANT) | (pos - (uint64_t(1) << T::MANT)));
    A x;
#ifdef __CUDA_ARCH__
    if constexpr (sizeof(A) == 8) x = __longlong_as_double((long long)b);
    else x = __uint_as_float(uint32_t(b));
#else
    std::memcpy(&x, &b, sizeof(A));
#endif
    return x;
}

// The grid position of a normal x of type A in its binade: its significand
// with the hidden bit.
template <class A>
QSLC_HD uint64_t grid_pos(A x)
{
    using T = fp_traits<A>;
    return (uint64_t(to_bits(x)) & ((uint64_t(1) << T::MANT) - 1)) | (uint64_t(1) << T::MANT);
}

// |a|^2 as the reference computes it: RN(RN(re*re) + RN(im*im))
// (measure.cpp:69-70, :141-142).
QSLC_HD double norm2_rn(double re, double im)
{
#ifdef __CUDA_ARCH__
    return __dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im));
#else
    volatile double a = re * re;   // volatile: no contraction on FMA hosts
    volatile double b = im * im;
    return a + b;
#endif
}
QSLC_HD float norm2_rn(float re, float im)
{
#ifdef __CUDA_ARCH__
    return __fadd_rn(__fmul_rn(re, re), __fmul_rn(im, im));
#else
    volatile float a = re * re;
    volatile float b = im * im;
    return a + b;
#endif
}

// Error-free double-double accumulation (Knuth's TwoSum); only an estimate
// of the exact prefix is needed, to guess each tile's binade.
struct dd {
    double hi, lo;
};
QSLC_HD dd dd_add(dd a, double b)
{
    double s = a.hi + b;
    double bb = s - a.hi;
    double err = (a.hi - (s - bb)) + (b - bb);
    double lo = a.lo + err;
    double hi = s + lo;
    return dd{hi, lo - (hi - s)};
}
QSLC_HD dd dd_add(dd a, dd b)
{
    dd r = dd_add(a, b.hi);
    r.lo += b.lo;
    double hi = r.hi + r.lo;
    return dd{hi, r.lo - (hi - r.hi)};
}

}  // namespace qslc
