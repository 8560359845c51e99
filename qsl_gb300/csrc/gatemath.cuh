// gatemath.cuh -- the arithmetic of one gate output, shared by the plain
// sweeps (gates.cu) and the number-preserving sweeps (np.cu).
//
// Every output is computed as the reference computes it, operation for
// operation, with each product and sum rounded on its own (no FMA).  For
// complex128 an output can instead run on the integer pipes through the
// exact binary64 emulation of dpemu.cuh; the bits are the same either way,
// and the split between the FP64 pipe and the integer pipes is chosen per
// sweep item by a pattern of masks.
#pragma once

#include "qslc_internal.cuh"
#include "dpemu.cuh"

#include <cmath>
#include <cstdlib>
#include <type_traits>

namespace qslc {

template <class T>
struct Coef {
    T c, s;  // cos/sin of angle/2 (rotations) or of angle (phase); sqrt2 for H
    emu::MulConst kc, ks;   // c and s decoded for the full integer path (double only)
    emu::MulK mc, ms;       // c and s decoded for the integer products of the mixed path
    emu::DivConst kd;       // c as a divisor (Hadamard)
};

// How one gate output RN(RN(a*k1) +- RN(b*k2)) is computed (complex128):
//   MD_F  both products and the sum on the FP64 pipe (3 FP64 operations);
//   MD_P  both products on the integer pipes (prod_pack), the sum on the
//        FP64 pipe (1 FP64 operation);
//   MD_Q  the first product on the integer pipes, the second product and the
//        sum on the FP64 pipe (2 FP64 operations);
//   MD_E  all of it on the integer pipes (dot2_rn, no FP64 operation).
// Every mode gives the reference's bits; they differ only in which pipes
// they load.  A mode mask holds 2 bits per output.
enum OutMode : unsigned { MD_F = 0, MD_P = 1, MD_Q = 2, MD_E = 3 };

// The FP64 fallbacks of the emulated outputs, out of line.  They run only
// for the operands the integer path declines (subnormals, infinities, NaNs,
// results outside the normal range).  Inline, a fallback of a few FP64
// instructions is cheap enough that the compiler predicates it instead of
// branching around it; predicated FP64 instructions still take their turn
// on the FP64 pipe, so every thread would pay for them and the emulation
// would save nothing.  A call is not turned into predicated arithmetic:
// measured on GB300, the inline forms ran the emulated patterns at the
// all-FP64 speed, the out-of-line form at the speed the pattern predicts.
template <bool NEG>
__device__ __noinline__ double dot2_fallback(double a, double k1, double b, double k2)
{
    return NEG ? __dsub_rn(__dmul_rn(a, k1), __dmul_rn(b, k2)) : __dadd_rn(__dmul_rn(a, k1), __dmul_rn(b, k2));
}
template <bool NEG>
__device__ __noinline__ double hdiv_fallback(double a, double b, double d)
{
    return __ddiv_rn(NEG ? __dsub_rn(a, b) : __dadd_rn(a, b), d);
}

// One Hadamard output, RN(RN(a +- b) / sqrt2) (gates.cpp:95-98).  The
// division always runs on the integer pipes (an FP64 divide is a long
// iteration on the FP64 pipe); with `em` set the sum does too.
template <class T, bool NEG>
__device__ __forceinline__ T hdiv(bool em, T a, T b, const Coef<T> &k)
{
    using R = rn<T>;
    if constexpr (sizeof(T) == 8) {
        bool ok = k.kd.usable != 0;
        if (ok) {
            uint64_t q;
            if (em) {
                const emu::Unp x = emu::unpack(emu::dbits(a), ok);
                emu::Unp y = emu::unpack(emu::dbits(b), ok);
                if (NEG) y.sign ^= emu::SIGN;
                q = emu::div_unp(emu::add_core(x, y, ok), k.kd, ok);
            } else {
                q = emu::div_fast(emu::dbits(NEG ? R::sub(a, b) : R::add(a, b)), k.kd, ok);
            }
            if (ok) return emu::dfrom(q);
        }
        return hdiv_fallback<NEG>(a, b, k.c);
    } else {
        return R::div(NEG ? R::sub(a, b) : R::add(a, b), k.c);
    }
}

// One output of a rotation or phase update: RN(RN(a*k1) + RN(b*k2)), or
// RN(RN(a*k1) - RN(b*k2)) when NEG.  With `em` set the integer pipes compute it
// (dpemu.cuh), falling back to the FP64 pipe for operands the integer path
// declines; either way the bits are the reference's.
template <class T, bool NEG>
__device__ __forceinline__ T dot2(bool em, T a, T k1, const emu::MulConst &e1, T b, T k2,
                                  const emu::MulConst &e2)
{
    if constexpr (sizeof(T) == 8) {
        if (em) {
            bool ok = (e1.usable & e2.usable) != 0;
            const uint64_t r = emu::dot2_rn(emu::dbits(a), e1, emu::dbits(b), e2, NEG, ok);
            if (ok) return emu::dfrom(r);
            return dot2_fallback<NEG>(a, k1, b, k2);
        }
    }
    using R = rn<T>;
    return NEG ? R::sub(R::mul(a, k1), R::mul(b, k2)) : R::add(R::mul(a, k1), R::mul(b, k2));
}

// One output in the given mode (see OutMode); `mode` must be the same
// across a warp.  Operands the integer products decline go to the FP64
// pipe out of line, as in dot2.
template <class T, bool NEG>
__device__ __forceinline__ T dot2m(unsigned mode, T a, T k1, const emu::MulConst &e1, const emu::MulK &m1,
                                   T b, T k2, const emu::MulConst &e2, const emu::MulK &m2)
{
    if constexpr (sizeof(T) == 8) {
        if (mode == MD_E) return dot2<T, NEG>(true, a, k1, e1, b, k2, e2);
        if (mode == MD_P) {
            bool ok = (m1.usable & m2.usable) != 0;
            const double p = emu::dfrom(emu::prod_pack(emu::dbits(a), m1, ok));
            const double q = emu::dfrom(emu::prod_pack(emu::dbits(b), m2, ok));
            if (ok) return NEG ? __dsub_rn(p, q) : __dadd_rn(p, q);
            return dot2_fallback<NEG>(a, k1, b, k2);
        }
        if (mode == MD_Q) {
            bool ok = m1.usable != 0;
            const double p = emu::dfrom(emu::prod_pack(emu::dbits(a), m1, ok));
            if (ok) {
                const double q = __dmul_rn(b, k2);
                return NEG ? __dsub_rn(p, q) : __dadd_rn(p, q);
            }
            return dot2_fallback<NEG>(a, k1, b, k2);
        }
    }
    using R = rn<T>;
    return NEG ? R::sub(R::mul(a, k1), R::mul(b, k2)) : R::add(R::mul(a, k1), R::mul(b, k2));
}

enum PairOp { P_SWAP, P_Y, P_H, P_RX, P_RY, P_RZ };
enum DiagOp { D_NEG, D_PHASE };

// Output i of a pair (r0.x, r0.y, r1.x, r1.y) takes mode (md >> 2i) & 3;
// Hadamard's sums run on the integer pipes for any mode but MD_F.  `md`
// must be the same across a warp.
__host__ __device__ constexpr unsigned mode_of(unsigned md, int i) { return (md >> (2 * i)) & 3u; }

template <class T, int OP>
__device__ __forceinline__ void pair_update(cplx<T> &a0, cplx<T> &a1, const Coef<T> &k, unsigned md = 0)
{
    using R = rn<T>;
    cplx<T> r0, r1;
    const unsigned E0 = mode_of(md, 0), E1 = mode_of(md, 1), E2 = mode_of(md, 2), E3 = mode_of(md, 3);
    if constexpr (OP == P_SWAP) {            // gates.cpp:41, :236, :524
        r0 = a1;
        r1 = a0;
    } else if constexpr (OP == P_Y) {        // gates.cpp:59-62, :267-270
        r0.x = a1.y; r0.y = -a1.x;
        r1.x = -a0.y; r1.y = a0.x;
    } else if constexpr (OP == P_H) {        // gates.cpp:95-98, :493-496, :675-678
        r0.x = hdiv<T, false>(E0 != MD_F, a0.x, a1.x, k);
        r0.y = hdiv<T, false>(E1 != MD_F, a0.y, a1.y, k);
        r1.x = hdiv<T, true>(E2 != MD_F, a0.x, a1.x, k);
        r1.y = hdiv<T, true>(E3 != MD_F, a0.y, a1.y, k);
    } else if constexpr (OP == P_RX) {       // gates.cpp:139-144, :336-341, :595-600
        r0.x = dot2m<T, false>(E0, a0.x, k.c, k.kc, k.mc, a1.y, k.s, k.ks, k.ms);
        r0.y = dot2m<T, true>(E1, a0.y, k.c, k.kc, k.mc, a1.x, k.s, k.ks, k.ms);
        r1.x = dot2m<T, false>(E2, a1.x, k.c, k.kc, k.mc, a0.y, k.s, k.ks, k.ms);
        r1.y = dot2m<T, true>(E3, a1.y, k.c, k.kc, k.mc, a0.x, k.s, k.ks, k.ms);
    } else if constexpr (OP == P_RY) {       // gates.cpp:169-174, :380-385, :638-643
        r0.x = dot2m<T, true>(E0, a0.x, k.c, k.kc, k.mc, a1.x, k.s, k.ks, k.ms);
        r0.y = dot2m<T, true>(E1, a0.y, k.c, k.kc, k.mc, a1.y, k.s, k.ks, k.ms);
        r1.x = dot2m<T, false>(E2, a0.x, k.s, k.ks, k.ms, a1.x, k.c, k.kc, k.mc);
        r1.y = dot2m<T, false>(E3, a0.y, k.s, k.ks, k.ms, a1.y, k.c, k.kc, k.mc);
    } else {                                 // P_RZ: gates.cpp:200-205, :424-429
        r0.x = dot2m<T, false>(E0, a0.x, k.c, k.kc, k.mc, a0.y, k.s, k.ks, k.ms);
        r0.y = dot2m<T, true>(E1, a0.y, k.c, k.kc, k.mc, a0.x, k.s, k.ks, k.ms);
        r1.x = dot2m<T, true>(E2, a1.x, k.c, k.kc, k.mc, a1.y, k.s, k.ks, k.ms);
        r1.y = dot2m<T, false>(E3, a1.y, k.c, k.kc, k.mc, a1.x, k.s, k.ks, k.ms);
    }
    a0 = r0;
    a1 = r1;
}

// Output i of a diagonal update (x, y) takes mode (md >> 2i) & 3.
template <class T, int OP>
__device__ __forceinline__ void diag_update(cplx<T> &a, const Coef<T> &k, unsigned md = 0)
{
    using R = rn<T>;
    if constexpr (OP == D_NEG) {             // gates.cpp:76-77, :296-297 (x *= -1)
        a.x = R::mul(a.x, T(-1));
        a.y = R::mul(a.y, T(-1));
    } else {                                 // gates.cpp:114-115, :460-461
        T x = a.x, y = a.y;
        a.x = dot2m<T, true>(mode_of(md, 0), x, k.c, k.kc, k.mc, y, k.s, k.ks, k.ms);
        a.y = dot2m<T, false>(mode_of(md, 1), y, k.c, k.kc, k.mc, x, k.s, k.ks, k.ms);
    }
}

// The old single-bit masks (bit i set: output i fully on the integer pipes)
// as a mode mask.
__host__ __device__ constexpr unsigned modes_from_bits(unsigned em)
{
    return ((em & 1u) ? 3u : 0u) | ((em & 2u) ? 12u : 0u) | ((em & 4u) ? 48u : 0u) | ((em & 8u) ? 192u : 0u);
}

// Bit insertion in the index type of a sweep: 32-bit arithmetic for states
// of up to 31 qubits (every index and shift then fits), 64-bit above.
template <class IX>
__host__ __device__ __forceinline__ IX ins0(IX j, unsigned t)
{
    const IX low = j & ((IX(1) << t) - 1);
    return ((j >> t) << (t + 1)) | low;
}
template <class IX>
__host__ __device__ __forceinline__ IX ins00(IX j, unsigned lo, unsigned hi)
{
    return ins0<IX>(ins0<IX>(j, lo), hi);
}

// The sweeps below take ITEMS work items per grid-stride iteration (at j,
// j + stride, j + 2 stride), all loads first.  `pat` holds one emulation
// mask per item, 4 bits each: item r uses (pat >> 4r) & 15, so the share of
// outputs computed on the integer pipes can be set in steps of one output
// in twelve (pair gates) or one in six (diagonal gates).  Masks differ only
// between items, never between threads of a warp.
#ifndef QSLC_ITEMS
#define QSLC_ITEMS 3
#endif
constexpr int ITEMS = QSLC_ITEMS;

// Launch bounds of the sweep kernels: 256 threads, and with QSLC_MINB set,
// at least that many resident CTAs per SM (which caps the registers).
#if defined(QSLC_MINB) && QSLC_MINB > 0
#define QSLC_SWEEP_BOUNDS __launch_bounds__(256, QSLC_MINB)
#else
#define QSLC_SWEEP_BOUNDS __launch_bounds__(256)
#endif

// A kernel's pattern is a template argument when it is one of the few
// compiled in (the mask tests then fold away, and so do the unused
// arithmetic paths and their registers); PAT_RUNTIME takes it from the
// kernel's argument instead, for any other setting.
constexpr unsigned PAT_RUNTIME = 0xFFFFFFFFu;

// The patterns compiled in: the defaults below and their neighbours, so a
// tuning sweep near the default measures compiled code too.  A pattern
// holds one 8-bit mode mask per sweep item (item r at bits 8r..8r+7), 2 bits
// per output (OutMode): e.g. 0x95 is P, P, P, Q for r0.x, r0.y, r1.x, r1.y,
// and 0x9 is P, Q for a diagonal update's x, y.
#ifndef QSLC_ROT_PATTERNS
#define QSLC_ROT_PATTERNS 0u, 0x959595u, 0xA59595u, 0x159595u, 0x999999u, 0x969696u, 0x151515u, 0xA5A5A5u, 0x033333u
#endif
#ifndef QSLC_ROT2_PATTERNS
#define QSLC_ROT2_PATTERNS 0u, 0x159595u, 0x959595u
#endif
#define QSLC_H_PATTERNS 0u, 0x000003u, 0x000303u
#ifndef QSLC_DIAG_PATTERNS
#define QSLC_DIAG_PATTERNS 0u, 0x090909u, 0x060606u, 0x010909u, 0x050909u, 0x030303u
#endif
#define QSLC_NP_PAIR_PATTERNS 0u, 0x030333u, 0x555555u, 0x959595u, 0xA5A5A5u
#define QSLC_NP_DIAG_PATTERNS 0u, 0x000303u, 0x050505u, 0x090909u, 0x0A0A0Au

// Launch `f(std::integral_constant<unsigned, P>{})` with P = pat when pat is
// one of CANDIDATES, else with PAT_RUNTIME.
template <unsigned... CANDIDATES, class F>
void with_pattern(unsigned pat, F &&f)
{
    bool done = false;
    ((pat == CANDIDATES && !done ? (f(std::integral_constant<unsigned, CANDIDATES>{}), done = true) : false),
     ...);
    if (!done) f(std::integral_constant<unsigned, PAT_RUNTIME>{});
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
    k.mc = emu::make_mulk(double(c));
    k.ms = emu::make_mulk(double(s));
    k.kd = emu::make_div(double(c));
    return k;
}
// The pattern a gate with coefficients k runs: `pat`, unless a coefficient
// is outside the integer products' range (an exact zero, a sine below
// 2^-64), where every output would decline to the FP64 pipe one by one --
// then all outputs run there from the start.
template <class T>
unsigned pattern_for(const Coef<T> &k, unsigned pat)
{
    return (k.mc.usable && k.ms.usable) ? pat : 0u;
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

// Share of the dense updates' work done on the integer pipes, as a pattern
// of one mode mask per sweep item (see ITEMS and OutMode).  The defaults
// balance the FP64 pipe against the integer pipes on GB300; environment
// variables override them for tuning: QSLC_EMU_MASK (rotations, one-qubit
// and controlled), QSLC_EMU_MASK_H (Hadamard), QSLC_EMU_MASK_DIAG (phase and
// controlPhase), QSLC_EMU_MASK_NP and QSLC_EMU_MASK_NP_DIAG (the
// number-preserving sweeps).  The value is one item ("PPPQ") or three
// ("PPPP,PPPP,PPPQ"), each a letter per output -- F, P, Q or E, as in
// OutMode -- or a decimal number in the older form (bit i set: output i
// fully on the integer pipes, mode E).  Items left out repeat the last one.
inline unsigned parse_item(const char *c, const char **endp, unsigned outputs, bool &good)
{
    unsigned md = 0;
    if (*c >= '0' && *c <= '9') {
        char *e = nullptr;
        const long v = std::strtol(c, &e, 10);
        *endp = e;
        if (v < 0 || v >= (1L << outputs)) good = false;
        return modes_from_bits(unsigned(v) & ((1u << outputs) - 1));
    }
    unsigned i = 0;
    for (; *c && *c != ','; c++, i++) {
        unsigned m;
        switch (*c) {
        case 'F': case 'f': m = MD_F; break;
        case 'P': case 'p': m = MD_P; break;
        case 'Q': case 'q': m = MD_Q; break;
        case 'E': case 'e': m = MD_E; break;
        default: m = MD_F; good = false; break;
        }
        if (i < outputs) md |= m << (2 * i);
        else good = false;
    }
    if (i == 0) good = false;
    *endp = c;
    return md;
}

inline unsigned parse_pattern(const char *var, const char *dflt, unsigned outputs)
{
    const char *e = std::getenv(var);
    unsigned m[3] = {0, 0, 0};   // three masks whatever ITEMS is; kernels use the first ITEMS
    for (int attempt = 0; attempt < 2; attempt++) {
        const char *src = (attempt == 0 && e && *e) ? e : dflt;
        bool good = true;
        int n = 0;
        for (const char *c = src; *c && n < 3;) {
            const char *endp = c;
            m[n++] = parse_item(c, &endp, outputs, good);
            if (*endp != ',') {
                if (*endp) good = false;
                break;
            }
            c = endp + 1;
        }
        if (n == 0) good = false;
        for (int i = n; i < 3; i++) m[i] = n ? m[n - 1] : 0;
        if (good) break;                 // a malformed override falls back to the default
    }
    return m[0] | (m[1] << 8) | (m[2] << 16);
}
inline unsigned pattern_rot()
{
    static unsigned p = parse_pattern("QSLC_EMU_MASK", "PPPQ,PPPQ,PPPF", 4);
    return p;
}
inline unsigned pattern_h()
{
    static unsigned p = parse_pattern("QSLC_EMU_MASK_H", "FFFF", 4);
    return p;
}
inline unsigned pattern_diag()
{
    static unsigned p = parse_pattern("QSLC_EMU_MASK_DIAG", "PQ,PQ,PP", 2);
    return p;
}
// The number-preserving sweeps spend integer work on ranking their indices,
// so their defaults differ: QSLC_EMU_MASK_NP (pair gates) and
// QSLC_EMU_MASK_NP_DIAG (single amplitudes).
inline unsigned pattern_np_pair()
{
    static unsigned p = parse_pattern("QSLC_EMU_MASK_NP", "PPPQ", 4);
    return p;
}
inline unsigned pattern_np_diag()
{
    static unsigned p = parse_pattern("QSLC_EMU_MASK_NP_DIAG", "PQ", 2);
    return p;
}

}  // namespace qslc
