// dpemu.cuh -- IEEE binary64 round-to-nearest-even multiply and add on the
// integer pipes.
//
// GB300 issues two FP64 operations per SM per clock against 64-128 integer
// operations.  qsl's gate loops round every product and every sum on its
// own (no FMA), so a dense gate costs 12 FP64 operations per amplitude pair,
// more than the FP64 pipe can retire at HBM speed.  These routines produce
// the same bits as __dmul_rn / __dadd_rn from integer arithmetic on the
// IEEE encodings, so a kernel can split its arithmetic between the FP64 pipe
// and the integer pipes.
//
// Coverage: finite normal operands and results, and zeros.  Anything else
// (subnormals, infinities, NaNs, a result that would overflow or underflow
// to a subnormal) reports `ok = false`, and the caller falls back to the
// native instruction, which is then exact by definition.
//
// Methods (textbook binary floating point, e.g. Muller et al., Handbook of
// Floating-Point Arithmetic, ch. 7-8):
//   mul: exact 106-bit product of the two 53-bit significands, then
//        round-to-nearest-even on the guard bit and a sticky bit.
//   add: align the smaller operand with guard bits, fold every shifted-out
//        bit into the least significant bit ("jamming"), add or subtract,
//        renormalise, round to nearest even on the guard bits.  The jammed
//        bit makes the computed sum odd whenever bits were dropped, so it
//        can never sit on a rounding tie and always rounds the way the exact
//        sum does.
//   div: quotient significand from a precomputed reciprocal of the constant
//        divisor, the rounding decided from the estimate's fraction bits,
//        and the few quotients too close to a midpoint declined.
// Kernels use the hot forms: dot2_rn (a rotation or phase output), div_fast
// (a Hadamard output), and add_core + div_unp (a Hadamard output with its
// sum on the integer pipes too).
#pragma once

#include <cstdint>
#include <cstring>

#include "replay.cuh"   // QSLC_HD

namespace qslc {
namespace emu {

constexpr uint64_t SIGN = 0x8000000000000000ull;
constexpr uint64_t MANT = 0x000FFFFFFFFFFFFFull;
constexpr uint64_t HIDDEN = 0x0010000000000000ull;

QSLC_HD uint64_t dbits(double x)
{
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    std::memcpy(&b, &x, 8);
    return b;
#endif
}

QSLC_HD double dfrom(uint64_t b)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double x;
    std::memcpy(&x, &b, 8);
    return x;
#endif
}

QSLC_HD uint64_t umulhi(uint64_t a, uint64_t b)
{
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

QSLC_HD int clz64(uint64_t x)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

// A multiplier fixed for a whole kernel (a gate coefficient), decoded once.
struct MulConst {
    uint64_t m;      // significand with the hidden bit, 53 bits
    int e;           // unbiased exponent
    uint64_t sign;   // SIGN or 0
    int usable;      // 0: zero/subnormal/inf/nan -- always use the native path
    uint32_t m0, m1; // m split into its low 32 and high 21 bits
    // biased exponents ef of a normal multiplicand for which a * c and its
    // rounding stay normal: ef - ef_lo <= ef_span (unsigned), one test
    uint32_t ef_lo, ef_span;
};

QSLC_HD MulConst make_const(double c)
{
    MulConst k{};
    const uint64_t b = dbits(c);
    const int ef = int((b >> 52) & 0x7FF);
    k.sign = b & SIGN;
    k.usable = (ef != 0 && ef != 0x7FF) ? 1 : 0;
    k.m = (b & MANT) | HIDDEN;
    k.e = ef - 1023;
    k.m0 = uint32_t(k.m);
    k.m1 = uint32_t(k.m >> 32);
    // product exponent ef - 1023 + e (+1 for a carry, +1 for a rounding
    // overflow) must stay in [-1022, 1023]
    const int lo = 1 - k.e > 1 ? 1 - k.e : 1;
    const int hi = 2044 - k.e < 2046 ? 2044 - k.e : 2046;
    if (lo > hi) k.usable = 0;
    // the dot product places a zero product at exponent -1023 + e, below
    // every normal product only while |c| < 2
    if (k.e > 0) k.usable = 0;
    k.ef_lo = uint32_t(lo);
    k.ef_span = lo > hi ? 0u : uint32_t(hi - lo);
    return k;
}

// mul_rn, add_rn and div_rn are the plain statements of the three
// operations, on 64-bit integers and with branches.  No kernel calls them;
// the CPU check holds them, and the hot forms further down, to the host's
// IEEE arithmetic.

// RN(a * c) for a normal constant c.  Zeros are exact; the rest needs a
// normal a and a normal result.
QSLC_HD uint64_t mul_rn(uint64_t a, const MulConst &c, bool &ok)
{
    const uint64_t sign = (a ^ c.sign) & SIGN;
    const uint64_t aa = a & ~SIGN;
    if (aa == 0) return sign;                       // +-0 * c
    const int ef = int(aa >> 52);
    if (ef == 0 || ef == 0x7FF) {
        ok = false;
        return 0;
    }
    const uint64_t ma = (aa & MANT) | HIDDEN;
    // 106-bit product ma * c.m in [2^104, 2^106): hi holds bits 64..105
    const uint64_t lo = ma * c.m;
    const uint64_t hi = umulhi(ma, c.m);
    const int top = int(hi >> 41) & 1;              // leading bit at 105?
    const int s = 52 + top;                         // bits below the kept 53
    uint64_t m = (hi << (64 - s)) | (lo >> s);
    const uint64_t rbit = (lo >> (s - 1)) & 1;
    const uint64_t sticky = lo & ((uint64_t(1) << (s - 1)) - 1);
    m += rbit & ((sticky != 0) | (m & 1));
    int e = ef - 1023 + c.e + top;
    if (m >> 53) {
        m >>= 1;
        e++;
    }
    if (e < -1022 || e > 1023) {
        ok = false;
        return 0;
    }
    return sign | (uint64_t(e + 1023) << 52) | (m & MANT);
}

// RN(x + y).
QSLC_HD uint64_t add_rn(uint64_t x, uint64_t y, bool &ok)
{
    uint64_t ax = x & ~SIGN, ay = y & ~SIGN;
    if (ax < ay) {
        uint64_t t = x; x = y; y = t;
        t = ax; ax = ay; ay = t;
    }
    if (ay == 0) {
        if (ax != 0) return x;                      // x + 0
        return x & y & SIGN;                        // +-0 + +-0: -0 only if both are
    }
    const int ex = int(ax >> 52), ey = int(ay >> 52);
    if (ex == 0x7FF || ey == 0) {                   // inf/nan, or a subnormal y (hence x too if ex == 0)
        ok = false;
        return 0;
    }
    const uint64_t X = ((ax & MANT) | HIDDEN) << 10;   // hidden bit at 62
    const uint64_t Yf = ((ay & MANT) | HIDDEN) << 10;
    const int d = ex - ey;
    uint64_t Y;
    if (d >= 63) {
        Y = 1;
    } else {
        Y = (Yf >> d) | (uint64_t((Yf & ((uint64_t(1) << d) - 1)) != 0));
    }
    uint64_t S;
    int e = ex;
    if (((x ^ y) & SIGN) == 0) {
        S = X + Y;
        if (S >> 63) {
            S = (S >> 1) | (S & 1);
            e++;
        }
    } else {
        S = X - Y;
        if (S == 0) return 0;                       // x - x = +0
        const int sh = clz64(S) - 1;
        S <<= sh;
        e -= sh;
    }
    uint64_t m = S >> 10;
    const uint64_t rb = S & 0x3FF;
    m += (rb > 0x200) | ((rb == 0x200) & (m & 1));
    if (m >> 53) {
        m >>= 1;
        e++;
    }
    if (e < 1 || e > 2046) {
        ok = false;
        return 0;
    }
    return (x & SIGN) | (uint64_t(e) << 52) | (m & MANT);
}

// A divisor fixed for a whole kernel (Hadamard's sqrt(2)), decoded once.
struct DivConst {
    uint64_t m;      // significand with the hidden bit
    uint64_t rinv;   // floor((2^116 - 1) / m): a 64-bit reciprocal
    uint32_t r0, r1, r2;   // floor((2^148 - 1) / m), below 2^96: a 96-bit reciprocal, low word first
    int e;           // unbiased exponent
    uint64_t sign;
    int usable;
    // biased exponents of a normal dividend whose quotient stays normal
    uint32_t ef_lo, ef_span;
};

inline DivConst make_div(double y)
{
    DivConst k{};
    uint64_t b;
    std::memcpy(&b, &y, 8);
    const int ef = int((b >> 52) & 0x7FF);
    k.sign = b & SIGN;
    k.usable = (ef != 0 && ef != 0x7FF) ? 1 : 0;
    k.m = (b & MANT) | HIDDEN;
    k.e = ef - 1023;
    const unsigned __int128 num = ((unsigned __int128)1 << 116) - 1;
    k.rinv = (uint64_t)(num / k.m);
    // 2^148 - 1 in base 2^32 is 0xFFFFF followed by four all-ones words;
    // long division by m keeps every partial remainder below 2^85
    unsigned __int128 rem = 0;
    uint32_t q[5];
    for (int i = 0; i < 5; i++) {
        const unsigned __int128 cur = (rem << 32) | (i == 0 ? 0xFFFFFu : 0xFFFFFFFFu);
        q[i] = uint32_t(cur / k.m);
        rem = cur % k.m;
    }
    k.r2 = q[2];
    k.r1 = q[3];
    k.r0 = q[4];
    if (q[0] | q[1]) k.usable = 0;   // cannot happen for m >= 2^52
    // quotient exponent ef - 1023 - e - (0 or 1) must stay in [-1021, 1022]
    const int lo = 3 + k.e > 1 ? 3 + k.e : 1;
    const int hi = 2045 + k.e < 2046 ? 2045 + k.e : 2046;
    if (lo > hi) k.usable = 0;
    k.ef_lo = uint32_t(lo);
    k.ef_span = lo > hi ? 0u : uint32_t(hi - lo);
    return k;
}

// RN(x / y), x packed, y a normal constant: the hot form of the division.
// With R = floor((2^148 - 1) / my), H = floor(mx * R / 2^32) is 2^116 * mx / my
// less under 2^22 + 1: the quotient significand t (53 bits, after one more
// left shift when mx < my) is its high part, and the next 64 bits v are the
// fraction that decides the rounding: up when v >= 2^63.  Only a fraction
// within 2^24 units of v of one half cannot be decided from the estimate
// (an exact tie always lands there); it declines (ok = false) and the
// caller divides on the FP64 pipe.  A fraction just below 1 whose true value
// crossed into the next integer rounds up to that integer either way.  The
// rounding increment goes into the packed result, so a carry moves into the
// exponent by itself.
QSLC_HD uint64_t div_fast(uint64_t x, const DivConst &y, bool &ok)
{
    const uint32_t xhi = uint32_t(x >> 32), xlo = uint32_t(x);
    const uint32_t ef = (xhi >> 20) & 0x7FF;
    const uint32_t sg = (xhi ^ uint32_t(y.sign >> 32)) & 0x80000000u;
    if (((xhi << 1) | xlo) == 0) return uint64_t(sg) << 32;     // +-0 / y
    ok = ok & ((ef - y.ef_lo) <= y.ef_span);
    const uint32_t m1 = (xhi & 0xFFFFFu) | 0x100000u, m0 = xlo;
    // H = a2:a1 words, high part hh: every partial sum below stays under 2^64
    const uint64_t s1 = uint64_t(m0) * y.r1 + ((uint64_t(m0) * y.r0) >> 32);
    const uint64_t t1 = uint64_t(m1) * y.r0;
    const uint64_t a1 = s1 + t1;
    const uint64_t k1 = uint64_t(a1 < t1);
    const uint64_t u = uint64_t(m0) * y.r2 + ((k1 << 32) | (a1 >> 32));
    const uint64_t t2 = uint64_t(m1) * y.r1;
    const uint64_t a2 = u + t2;
    const uint64_t k2 = uint64_t(a2 < t2);
    const uint64_t hh = uint64_t(m1) * y.r2 + ((k2 << 32) | (a2 >> 32));
    const uint64_t hl = (a2 << 32) | (a1 & 0xFFFFFFFFu);
    const uint64_t k53 = uint64_t(hh < HIDDEN);
    const uint64_t t = (hh << k53) | ((hl >> 63) & k53);
    const uint64_t v = hl << k53;
    ok = ok & (((v ^ SIGN) + (uint64_t(1) << 24)) >= (uint64_t(1) << 25));
    const int E = int(ef) - 1023 - y.e - int(k53);
    return (uint64_t(sg) << 32) | ((uint64_t(uint32_t(E + 1022)) << 52) + t + (v >> 63));
}

// RN(x / y) for a normal constant y.  The quotient significand
// t = floor(mx * 2^k / my) (k = 52 or 53 so that t has 53 bits) is
// estimated with the reciprocal, which is low by at most one, corrected with
// the exact remainder r = mx * 2^k - t * my (below 2 * my, so its low 64
// bits are the whole of it), and rounded to nearest even by comparing 2r
// with my.
QSLC_HD uint64_t div_rn(uint64_t x, const DivConst &y, bool &ok)
{
    const uint64_t sign = (x ^ y.sign) & SIGN;
    const uint64_t ax = x & ~SIGN;
    if (ax == 0) return sign;
    const int ef = int(ax >> 52);
    if (ef == 0 || ef == 0x7FF) {
        ok = false;
        return 0;
    }
    const uint64_t mx = (ax & MANT) | HIDDEN;
    const int k = mx >= y.m ? 52 : 53;
    const uint64_t hi = umulhi(mx, y.rinv), lo = mx * y.rinv;
    uint64_t t = (k == 52) ? hi : ((hi << 1) | (lo >> 63));
    uint64_t r = (mx << k) - t * y.m;             // exact: the true remainder < 2^54
    if (r >= y.m) {
        t++;
        r -= y.m;
    }
    const uint64_t r2 = r << 1;
    t += (r2 > y.m) | ((r2 == y.m) & (t & 1));
    int e = ef - 1023 - y.e - k + 52;
    if (t >> 53) {
        t >>= 1;
        e++;
    }
    if (e < -1022 || e > 1023) {
        ok = false;
        return 0;
    }
    return sign | (uint64_t(e + 1023) << 52) | (t & MANT);
}

// ---------------------------------------------------------------------------
// The unpacked path of a Hadamard output whose sum also runs on the integer
// pipes: RN(RN(a +- b) / y) as div_unp(add_core(unpack(a), unpack(+-b))),
// with the sum handed to the division unpacked -- sign, exponent, 53-bit
// significand -- instead of packed into IEEE bits and unpacked again.
// ---------------------------------------------------------------------------

// value = m * 2^(e - 52) with m in [2^52, 2^53), or zero when m == 0
struct Unp {
    uint64_t m;
    int e;
    uint64_t sign;   // SIGN or 0
};

// IEEE bits to the unpacked form; declines subnormals, infinities, NaNs.
QSLC_HD Unp unpack(uint64_t a, bool &ok)
{
    Unp r;
    r.sign = a & SIGN;
    const uint32_t ahi = uint32_t(a >> 32);
    const int ef = int((ahi >> 20) & 0x7FF);
    if (((ahi & 0x7FFFFFFFu) | uint32_t(a)) == 0) {
        r.m = 0;
        r.e = 0;
        return r;
    }
    ok = ok & (ef != 0) & (ef != 0x7FF);
    r.m = (a & MANT) | HIDDEN;
    r.e = ef - 1023;
    return r;
}

// RN(x + y) of two unpacked values, still unpacked (a zero keeps its sign).
QSLC_HD Unp add_core(Unp x, Unp y, bool &ok)
{
    const uint64_t kx = x.m ? (uint64_t(x.e + 1100) << 53) | x.m : 0;
    const uint64_t ky = y.m ? (uint64_t(y.e + 1100) << 53) | y.m : 0;
    if (kx < ky) {
        const Unp t = x;
        x = y;
        y = t;
    }
    const uint64_t X = x.m << 10, Yf = y.m << 10;   // lead bit at 62, 10 guard bits
    int d = x.e - y.e;
    d = d < 0 ? 0 : (d > 63 ? 63 : d);              // d < 0 only when y is zero
    const uint64_t Y = (Yf >> d) | uint64_t((Yf & ((uint64_t(1) << d) - 1)) != 0);
    const bool sub = (x.sign ^ y.sign) != 0;
    uint64_t S = sub ? X - Y : X + Y;
    Unp r;
    if (S == 0) {                                   // exact cancellation: +0; 0 + 0 keeps a shared sign
        r.m = 0;
        r.e = 0;
        r.sign = sub ? 0 : (x.sign & y.sign);
        return r;
    }
    const int lz = clz64(S);
    int e = x.e;
    if (lz == 0) {                                  // carry out of an addition
        S = (S >> 1) | (S & 1);
        e += 1;
    } else {
        S <<= (lz - 1);
        e -= lz - 1;
    }
    uint64_t m = S >> 10;
    const uint64_t rb = S & 0x3FF;
    m += uint64_t(rb > 0x200) | (uint64_t(rb == 0x200) & (m & 1));
    const uint64_t carry = m >> 53;
    m >>= carry;
    e += int(carry);
    ok = ok & (e >= -1022) & (e <= 1023);
    r.m = m;
    r.e = e;
    r.sign = x.sign;
    return r;
}

// RN(x / y) for an unpacked x and a normal constant y, packed.  The
// quotient significand t = floor(mx * 2^k / my) (k = 52 when mx >= my, else
// 53, so that t has 53 bits) is estimated from the high part of mx times the
// 64-bit reciprocal, leaving out the low 32 x 32 partial product; the
// estimate is then low by at most three (one from the reciprocal, two from
// the dropped part when k = 53).  The exact remainder
// r = mx * 2^k - t * my (its low 64 bits are all of it) corrects it, and
// comparing 2r with my rounds to nearest even.
QSLC_HD uint64_t div_unp(const Unp &x, const DivConst &y, bool &ok)
{
    const uint64_t sign = x.sign ^ y.sign;
    if (x.m == 0) return sign;
    const uint64_t mx = x.m;
    const uint32_t m0 = uint32_t(mx), m1 = uint32_t(mx >> 32);
    const uint32_t r0 = uint32_t(y.rinv), r1 = uint32_t(y.rinv >> 32);
    const uint64_t a = uint64_t(m0) * r1, b = uint64_t(m1) * r0;
    const uint64_t mid = a + b;
    const uint64_t midc = uint64_t(mid < a);       // carry out of the 64-bit sum
    const uint64_t hi = uint64_t(m1) * r1 + (mid >> 32) + (midc << 32);
    const uint64_t k53 = uint64_t(mx < y.m);
    uint64_t t = (hi << k53) | ((mid >> 31) & k53);  // bit 63 of the truncated product is bit 31 of mid
    uint64_t r = (mx << (52 + k53)) - t * y.m;
#pragma unroll
    for (int step = 0; step < 3; step++) {
        const bool c = r >= y.m;
        t += c ? 1 : 0;
        r -= c ? y.m : 0;
    }
    const uint64_t r2 = r << 1;
    t += uint64_t(r2 > y.m) | (uint64_t(r2 == y.m) & (t & 1));
    int e = x.e - y.e - int(k53);
    const uint64_t carry = t >> 53;
    t >>= carry;
    e += int(carry);
    ok = ok & (e >= -1022) & (e <= 1023);
    return sign | (uint64_t(e + 1023) << 52) | (t & MANT);
}

// RN(RN(a*c) + RN(b*s)), or RN(RN(a*c) - RN(b*s)) when neg: the shape of
// every rotation and phase output in qsl's gate loops (e.g. a0.real*cos +
// a1.imag*sin, gates.cpp:139).  `ok` reports whether the integer path
// covered every step; when it did not, the result is meaningless.
//
// The code below is the hot form, written for 32-bit integer pipes:
//  - a product is RN(a * c) with its significand left unnormalised when the
//    rounding carries out (m = 2^53 then stands for 2^52 at exponent + 1).
//    A zero has no hidden bit, so its product is m = 0 by itself, with the
//    exponent -1023 + e(c), below that of every normal product because
//    |c| < 2 (make_const declines larger constants);
//  - the sum orders its operands by exponent, then significand, so the
//    larger one comes first and a subtraction never comes out negative;
//  - it normalises by a single left shift by the count of leading zeros,
//    which also covers the carry of an addition;
//  - the rounding increment is added to the packed result, so a carry out
//    of the significand moves into the exponent field by itself.
// Operands outside the normal range (or whose products or sum would leave
// it) set ok = false.

// RN(a * c): significand (53 bits, or 2^53; 0 for a zero), exponent, sign
// in bit 31.
QSLC_HD void prod_fast(uint64_t a, const MulConst &c, uint64_t &m, int &e, uint32_t &sg, bool &ok)
{
    const uint32_t ahi = uint32_t(a >> 32), alo = uint32_t(a);
    const uint32_t ef = (ahi >> 20) & 0x7FF;
    sg = (ahi ^ uint32_t(c.sign >> 32)) & 0x80000000u;
    const bool zero = ((ahi << 1) | alo) == 0;
    ok = ok & (zero | ((ef - c.ef_lo) <= c.ef_span));
    const uint32_t a1 = (ahi & 0xFFFFFu) | (ef ? 0x100000u : 0u);
    const uint64_t p00 = uint64_t(alo) * c.m0, p01 = uint64_t(alo) * c.m1;
    const uint64_t p10 = uint64_t(a1) * c.m0, p11 = uint64_t(a1) * c.m1;
    const uint64_t mid = p01 + p10;
    const uint64_t lo = p00 + (mid << 32);
    const uint64_t hi = p11 + (mid >> 32) + uint64_t(lo < p00);   // product = hi:lo < 2^106
    const uint32_t top = uint32_t(hi >> 41);
    uint64_t q = (hi << 13) | (lo >> 51);                          // product >> 51
    uint64_t st = uint64_t((lo & ((uint64_t(1) << 51) - 1)) != 0);
    st |= q & top;
    q >>= top;
    uint64_t mm = q >> 1;
    mm += (q & 1) & (st | (mm & 1));
    m = mm;
    e = int(ef) - 1023 + c.e + int(top);
}

QSLC_HD uint64_t dot2_rn(uint64_t a, const MulConst &c, uint64_t b, const MulConst &s, bool neg,
                         bool &ok)
{
    uint64_t mp, mq;
    int ep, eq;
    uint32_t sp, sq;
    prod_fast(a, c, mp, ep, sp, ok);
    prod_fast(b, s, mq, eq, sq, ok);
    if (neg) sq ^= 0x80000000u;
    // x: the larger operand
    const bool sw = (eq > ep) | ((eq == ep) & (mq > mp));
    const uint64_t mx = sw ? mq : mp, my = sw ? mp : mq;
    const int ex = sw ? eq : ep, ey = sw ? ep : eq;
    const uint32_t sx = sw ? sq : sp;
    // lead bit at 60 (61 for 2^53), so even the sum of two products that both
    // rounded up to 2^53 stays below 2^63; with at least 8 trailing zeros in
    // both, no bit is dropped unless d > 8, and then the result keeps its
    // lead within one place of bit 60
    const uint64_t X = mx << 8, Yf = my << 8;
    const unsigned dd = unsigned(ex - ey);
    const unsigned d = dd > 63 ? 63 : dd;
    const uint64_t Y = (Yf >> d) | uint64_t((Yf & ((uint64_t(1) << d) - 1)) != 0);
    const bool sub = ((sp ^ sq) & 0x80000000u) != 0;
    const uint64_t S = sub ? X - Y : X + Y;
    if (S == 0) return uint64_t(sub ? 0u : (sp & sq)) << 32;
    const int lz = clz64(S);                        // >= 1: S <= 2^61 + 2^61
    const uint64_t N = S << lz;                     // lead bit at 63
    const int E = ex + 3 - lz;
    const uint64_t mr = N >> 11;
    // round to nearest even on the 11 bits below: carry out of rb + 0x3FF + lsb
    const uint32_t rb = uint32_t(N) & 0x7FFu;
    const uint32_t inc = (rb + 0x3FFu + (uint32_t(mr) & 1u)) >> 11;
    ok = ok & (E >= -1021) & (E <= 1022);
    return (uint64_t(sx) << 32) | ((uint64_t(uint32_t(E + 1022)) << 52) + mr + inc);
}

// ---------------------------------------------------------------------------
// RN(a * c) as packed IEEE bits from 32-bit integer work: the product form
// of the mixed path, where a gate output RN(RN(a*c) + RN(b*s)) takes its
// products from the integer pipes and its sum from the FP64 pipe (one FP64
// operation instead of three).
//
// The constant's significand is stored shifted left by 11 (C = mc * 2^11,
// bit 63 set), so the 128-bit product P = ma * C lies in [2^115, 2^117)
// and the 53 bits it keeps start at bit 64 (or 63): the significand is the
// high 64-bit word, or that word and one more bit, and the bits below it are
// whole 32-bit words.  The four 32 x 32 partial products are
// multiply-adds whose carries never leave 64 bits (they run on the FMA
// pipe's IMAD.WIDE); the rest is a handful of 32-bit shifts, logic and
// adds:
//   - top = bit 116 of P; a funnel shift by 1 - top brings the significand
//     to 53 bits and leaves the round bit at bit 31 of `rest`;
//   - the lowest word is jammed into rest's last bit, so the round-to-
//     nearest-even increment is the carry out of rest + 0x7FFFFFFF + lsb;
//   - the significand (hidden bit included) is added to the sign and the
//     exponent field less one, so the hidden bit -- or a rounding carry to
//     2^53 -- moves into the exponent by itself.
// A zero a gives a zero of the product's sign.  Subnormal, infinite or NaN
// operands, and products whose exponent would leave the normal range, set
// ok = false; the caller then multiplies on the FP64 pipe.
// ---------------------------------------------------------------------------

// A multiplier fixed for a whole kernel, decoded for prod_pack.  Only
// constants with 2^-64 <= |c| < 2 are usable (every rotation and phase
// coefficient but an exact zero or a sine below 2^-64); the accepted
// multiplicands then do not depend on the constant -- exponent fields 65 to
// 2044, whose products with any usable constant are normal even after a
// rounding carry -- so the two products of one operand share that test.
struct MulK {
    uint32_t c0, c1;      // mc * 2^11 = c1:c0
    uint32_t ehi;         // (e(c) - 1) << 20, two's complement
    uint32_t sign;        // sign of c in bit 31
    int usable;           // 0: c outside [2^-64, 2) in magnitude, or not finite
};

constexpr uint32_t PACK_EF_LO20 = 65u << 20;              // lowest accepted exponent field, << 20
constexpr uint32_t PACK_EF_SPAN20 = (2044u - 65u) << 20;  // accepted span, << 20

QSLC_HD MulK make_mulk(double c)
{
    const MulConst k = make_const(c);
    MulK r{};
    const uint64_t C = k.m << 11;
    r.c0 = uint32_t(C);
    r.c1 = uint32_t(C >> 32);
    r.ehi = uint32_t(k.e - 1) << 20;
    r.sign = uint32_t(k.sign >> 32);
    // product exponent field ef + e(c) + top (+1 after a rounding carry)
    // stays in [1, 2046] for ef in [65, 2044] when e(c) is in [-64, 0]
    const int ef = int((dbits(c) >> 52) & 0x7FF);
    r.usable = (ef != 0 && ef != 0x7FF && k.e >= -64 && k.e <= 0) ? 1 : 0;
    return r;
}

QSLC_HD uint32_t fshl1(uint32_t lo, uint32_t hi, uint32_t s)   // (hi:lo) << s >> 32, s in {0, 1}
{
#ifdef __CUDA_ARCH__
    return __funnelshift_l(lo, hi, s);
#else
    return (hi << s) | ((lo >> 31) & s);
#endif
}

QSLC_HD uint64_t mulwide(uint32_t a, uint32_t b) { return uint64_t(a) * b; }

// (mh:ml:rest) + k as a 96-bit add, returning the top two words with e
// added to the top one: one carry chain.
QSLC_HD void add96(uint32_t mh, uint32_t ml, uint32_t rest, uint32_t k, uint32_t e, uint32_t &hi,
                   uint32_t &lo)
{
#ifdef __CUDA_ARCH__
    // the first add only makes the carry; its sum lands in lo, which the
    // second add overwrites
    asm("add.cc.u32 %0, %2, %3;\n\t"
        "addc.cc.u32 %0, %4, 0;\n\t"
        "addc.u32 %1, %5, %6;"
        : "=&r"(lo), "=r"(hi)
        : "r"(rest), "r"(k), "r"(ml), "r"(mh), "r"(e));
#else
    const uint64_t t0 = uint64_t(rest) + k;
    const uint64_t t1 = uint64_t(ml) + (t0 >> 32);
    lo = uint32_t(t1);
    hi = mh + e + uint32_t(t1 >> 32);
#endif
}

// Per-operand part of prod_pack, shared by the operand's products with
// different constants.
struct PackOp {
    uint32_t alo, a1;     // significand: a1 (hidden bit unless zero) : alo
    uint32_t efield;      // exponent field, in place (<< 20)
    uint32_t ahi;         // sign source
    bool zero;
};

QSLC_HD PackOp pack_operand(uint64_t abits, bool &ok)
{
    PackOp o;
    o.ahi = uint32_t(abits >> 32);
    o.alo = uint32_t(abits);
    o.efield = o.ahi & 0x7FF00000u;
    o.zero = ((o.ahi & 0x7FFFFFFFu) | o.alo) == 0;
    ok = ok & (o.zero | ((o.efield - PACK_EF_LO20) <= PACK_EF_SPAN20));
    o.a1 = (o.ahi & 0x000FFFFFu) | (o.zero ? 0u : 0x00100000u);
    return o;
}

QSLC_HD uint64_t prod_pack_op(const PackOp &o, const MulK &k)
{
    // P = (a1:alo) * (c1:c0) = w3:w2:w1:w0, in [2^115, 2^117) (0 for a zero)
    const uint64_t p00 = mulwide(o.alo, k.c0);
    const uint64_t p01 = mulwide(o.alo, k.c1) + (p00 >> 32);
    const uint64_t p10 = mulwide(o.a1, k.c0) + uint32_t(p01);
    const uint64_t p11 = mulwide(o.a1, k.c1) + (p01 >> 32) + (p10 >> 32);
    const uint32_t w0 = uint32_t(p00), w1 = uint32_t(p10);
    const uint32_t w2 = uint32_t(p11), w3 = uint32_t(p11 >> 32);
    const uint32_t top20 = w3 & 0x00100000u;          // bit 116 of P, in place
    const uint32_t sg = (o.ahi ^ k.sign) & 0x80000000u;
    // exponent field less one (the hidden bit adds it back), sign; a zero
    // keeps only its sign
    const uint32_t e = (o.zero ? 0u : o.efield + k.ehi + top20) | sg;
    uint32_t hi, lo;
    const uint32_t s = (top20 >> 20) ^ 1u;
    const uint32_t mh = fshl1(w2, w3, s), ml = fshl1(w1, w2, s);
    // c0 has 11 trailing zeros, so w0 does too: w0 >> 11 is nonzero exactly
    // when w0 is, and lands below the round bit as the sticky bits
    const uint32_t rest = (w1 << s) | (w0 >> 11);
    // round to nearest even: the carry out of rest + 0x7FFFFFFF + lsb
    const uint32_t kround = 0x7FFFFFFFu + (ml & 1u);
    add96(mh, ml, rest, kround, e, hi, lo);
    return (uint64_t(hi) << 32) | lo;
}

// RN(a * c) packed, or ok = false when a or the result is outside the
// covered range (see MulK); the caller then multiplies on the FP64 pipe.
QSLC_HD uint64_t prod_pack(uint64_t abits, const MulK &k, bool &ok)
{
    const PackOp o = pack_operand(abits, ok);
    return prod_pack_op(o, k);
}

}  // namespace emu
}  // namespace qslc
