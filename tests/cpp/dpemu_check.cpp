// Checks the integer-pipe binary64 arithmetic (qsl_gb300/csrc/dpemu.cuh)
// against the host's IEEE multiply and add, bit for bit.  Operands mix
// random significands with significands that have few set bits (which make
// exact products, exact sums and rounding ties common), exponent gaps from 0
// to 70, both signs, zeros, and results near the overflow and underflow
// thresholds (where the routines must either be exact or decline).
#include "dpemu.cuh"

#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <random>

using namespace qslc::emu;

static std::mt19937_64 rng(12345);

static double make(int emin, int emax)
{
    uint64_t m = rng() & MANT;
    switch (rng() % 4) {
    case 0: m &= ~((uint64_t(1) << (rng() % 53)) - 1); break;        // trailing zeros
    case 1: m = (rng() % 64) << (rng() % 46); m &= MANT; break;         // few bits
    default: break;
    }
    int e = emin + int(rng() % uint64_t(emax - emin + 1));
    uint64_t b = (uint64_t(e + 1023) << 52) | m | (rng() & 1 ? SIGN : 0);
    return dfrom(b);
}

// A significand ma in [2^52, 2^53) whose product with mc rounds up to the
// next power of two: ma * mc in [2^105 - 2^51, 2^105) (top = 0) or in
// [2^106 - 2^52, 2^106) (top = 1).  Not every mc has one.
static bool carry_significand(uint64_t mc, int top, uint64_t &ma)
{
    typedef unsigned __int128 u128;
    const u128 hi = u128(1) << (105 + top);
    const u128 lo = hi - (u128(1) << (51 + top));
    const u128 m = (lo + mc - 1) / mc;
    if (m < HIDDEN || m >= 2 * HIDDEN || m * mc >= hi) return false;
    ma = uint64_t(m);
    return true;
}

// x^-1 mod m for x coprime to m (extended Euclid; m < 2^53).
static uint64_t inverse_mod(uint64_t x, uint64_t m)
{
    int64_t r0 = int64_t(m), r1 = int64_t(x % m), t0 = 0, t1 = 1;
    while (r1 != 0) {
        const int64_t q = r0 / r1, r2 = r0 - q * r1, t2 = t0 - q * t1;
        r0 = r1; r1 = r2; t0 = t1; t1 = t2;
    }
    return uint64_t(t0 < 0 ? t0 + int64_t(m) : t0);
}

// Dividends whose quotient by y sits next to a rounding decision: with
// my odd and k = 52 (mx >= my) or 53 (mx < my), the significand mx with
// mx * 2^k = r (mod my) leaves the fraction r / my: (my -+ 1) / 2 put it
// 1 / (2 my) from one half, 0 makes the quotient exact, my - 1 puts it just
// below the next integer.  The division must decline the first two (no
// estimate decides them) and get every decided one right.
static long near_midpoint_cases(double yv, long &declined, long &fails)
{
    const DivConst kd = make_div(yv);
    const uint64_t my = kd.m;
    long n = 0;
    for (int k53 = 0; k53 < 2; k53++) {
        const uint64_t inv = inverse_mod((uint64_t(1) << (52 + k53)) % my, my);
        const uint64_t rs[5] = {(my - 1) / 2, (my + 1) / 2, 0, my - 1, 1};
        for (int ri = 0; ri < 5; ri++) {
            const uint64_t mx0 = uint64_t((unsigned __int128)rs[ri] * inv % my);
            for (uint64_t j = 0; j < 4; j++) {
                const uint64_t mx = mx0 + j * my;
                if (mx < HIDDEN || mx >= 2 * HIDDEN || (mx < my) != (k53 == 1)) continue;
                for (int e = -30; e <= 2; e += 4) {
                    for (int sgn = 0; sgn < 2; sgn++) {
                        const double xv = std::ldexp(double(mx), e - 52) * (sgn ? -1.0 : 1.0);
                        volatile double qref = xv / yv;
                        bool ok = true;
                        const uint64_t q = div_fast(dbits(xv), kd, ok);
                        n++;
                        if (!ok) declined++;
                        if (ok && q != dbits(qref)) {
                            if (fails++ < 10)
                                std::printf("div_fast near midpoint %a / %a: got %a want %a\n", xv, yv,
                                            dfrom(q), (double)qref);
                        }
                        if (ri < 2 && ok) {
                            if (fails++ < 10) std::printf("div_fast decided a midpoint case %a / %a\n", xv, yv);
                        }
                        bool ok2 = true;
                        const uint64_t q2 = div_unp(unpack(dbits(xv), ok2), kd, ok2);
                        if (ok2 && q2 != dbits(qref)) {
                            if (fails++ < 10)
                                std::printf("div_unp near midpoint %a / %a: got %a want %a\n", xv, yv,
                                            dfrom(q2), (double)qref);
                        }
                    }
                }
            }
        }
    }
    return n;
}

int main(int argc, char **argv)
{
    const long N = argc > 1 ? std::atol(argv[1]) : 20000000;
    long fails = 0, declined_mul = 0, declined_add = 0, declined_dot = 0, declined_div = 0;
    for (long i = 0; i < N; i++) {
        // multiply: constant-like c, amplitude-like a, plus edge exponents
        double c = (i & 7) == 0 ? make(-1022, 1023) : make(-6, 1);
        double a = (i & 7) == 1 ? make(-1022, 1023) : make(-80, 2);
        if ((i & 255) == 3) a = (rng() & 1) ? 0.0 : -0.0;
        MulConst k = make_const(c);
        bool ok = true;
        uint64_t r = mul_rn(dbits(a), k, ok);
        volatile double ref = a * c;
        if (ok && r != dbits(ref)) {
            if (fails++ < 10)
                std::printf("mul %a * %a: got %a want %a\n", a, c, dfrom(r), (double)ref);
        }
        if (!ok) declined_mul++;
        // add: exponent gap 0..70, both signs
        double x = make(-60, 3);
        int gap = int(rng() % 71);
        uint64_t xb = dbits(x);
        int ex = int((xb >> 52) & 0x7FF) - 1023;
        int ey = ex - gap + int(rng() % 3) - 1;
        if (ey < -1022) ey = -1022;
        double y = make(ey, ey);
        if ((i & 255) == 5) y = (rng() & 1) ? 0.0 : -0.0;
        if ((i & 255) == 6) y = -x;
        if ((i & 1023) == 7) { x = make(1020, 1023); y = make(1020, 1023); }   // overflow region
        if ((i & 1023) == 8) { x = make(-1022, -1020); y = -make(-1022, -1020); } // underflow region
        ok = true;
        uint64_t s = add_rn(dbits(x), dbits(y), ok);
        volatile double sref = x + y;
        if (ok && s != dbits(sref)) {
            if (fails++ < 10)
                std::printf("add %a + %a: got %a want %a\n", x, y, dfrom(s), (double)sref);
        }
        if (!ok) declined_add++;
        // division by a constant: sqrt(2) (Hadamard) and random divisors
        {
            double yv = (i & 3) ? 1.4142135623730951 : make(-8, 8);
            DivConst kd = make_div(yv);
            double xv = (i & 15) == 9 ? make(-1022, 1023) : make(-80, 3);
            if ((i & 255) == 10) xv = (rng() & 1) ? 0.0 : -0.0;
            ok = true;
            uint64_t qd = div_rn(dbits(xv), kd, ok);
            volatile double qref = xv / yv;
            if (ok && qd != dbits(qref)) {
                if (fails++ < 10) std::printf("div %a / %a: got %a want %a\n", xv, yv, dfrom(qd), (double)qref);
            }
            // the hot form of the division
            {
                bool ok5 = kd.usable != 0;
                const uint64_t qf = div_fast(dbits(xv), kd, ok5);
                if (ok5 && qf != dbits(qref)) {
                    if (fails++ < 10)
                        std::printf("div_fast %a / %a: got %a want %a\n", xv, yv, dfrom(qf), (double)qref);
                }
                if (!ok5) declined_div++;
            }
            // the unpacked division must agree with the packed one bit for bit
            {
                bool ok2 = kd.usable != 0;
                const Unp ux = unpack(dbits(xv), ok2);
                const uint64_t qu = div_unp(ux, kd, ok2);
                if (ok2 && qu != dbits(qref)) {
                    if (fails++ < 10)
                        std::printf("div_unp %a / %a: got %a want %a\n", xv, yv, dfrom(qu), (double)qref);
                }
                if (!ok2) declined_div++;
            }
            // a Hadamard output, RN(RN(a +- b) / sqrt2), with the sum unpacked
            {
                const double ha = make(-60, 1), hb = (i & 7) == 3 ? ha : make(-62, 1);
                const bool hneg = rng() & 1;
                bool ok3 = kd.usable != 0;
                const Unp sa = unpack(dbits(ha), ok3);
                Unp sb = unpack(dbits(hb), ok3);
                if (hneg) sb.sign ^= SIGN;
                const uint64_t hq = div_unp(add_core(sa, sb, ok3), kd, ok3);
                volatile double hs = hneg ? ha - hb : ha + hb;
                volatile double href = hs / yv;
                if (ok3 && hq != dbits(href)) {
                    if (fails++ < 10)
                        std::printf("hdiv (%a %c %a) / %a: got %a want %a\n", ha, hneg ? '-' : '+', hb, yv,
                                    dfrom(hq), (double)href);
                }
            }
            // exact quotients and exact halfway cases: x = q * y for short q
            double qv = make(-4, 4);
            double prod = qv * yv;
            ok = true;
            qd = div_rn(dbits(prod), kd, ok);
            volatile double qref2 = prod / yv;
            if (ok && qd != dbits(qref2)) {
                if (fails++ < 10) std::printf("div2 %a / %a: got %a want %a\n", prod, yv, dfrom(qd), (double)qref2);
            }
            bool ok6 = kd.usable != 0;
            const uint64_t qf2 = div_fast(dbits(prod), kd, ok6);
            if (ok6 && qf2 != dbits(qref2)) {
                if (fails++ < 10)
                    std::printf("div_fast2 %a / %a: got %a want %a\n", prod, yv, dfrom(qf2), (double)qref2);
            }
            bool ok4 = kd.usable != 0;
            const uint64_t qu2 = div_unp(unpack(dbits(prod), ok4), kd, ok4);
            if (ok4 && qu2 != dbits(qref2)) {
                if (fails++ < 10)
                    std::printf("div_unp2 %a / %a: got %a want %a\n", prod, yv, dfrom(qu2), (double)qref2);
            }
        }
        // the fused shape of a rotation output, RN(RN(a*c) +- RN(b*s)), with
        // the operand mixes a gate sees: amplitude-like values, zeros,
        // near-cancellation (b*s close to a*c), wide exponent gaps
        for (int rep = 0; rep < 2; rep++) {
            double a2 = make(-80, 2), c2 = make(-6, 0), b2 = make(-80, 2), s2 = make(-6, 0);   // |c| < 2, like gate constants
            const int kind = int(rng() % 8);
            if (kind == 0) a2 = (rng() & 1) ? 0.0 : -0.0;
            if (kind == 1) b2 = (rng() & 1) ? 0.0 : -0.0;
            if (kind == 2) { a2 = (rng() & 1) ? 0.0 : -0.0; b2 = (rng() & 1) ? 0.0 : -0.0; }
            if (kind == 3) { b2 = a2; s2 = c2; }                                  // exact cancellation
            if (kind == 4) { b2 = dfrom(dbits(a2) + (rng() % 5) - 2); s2 = c2; }   // near cancellation
            if (kind == 5) { b2 = make(-1022, -900); }                             // tiny second term
            if (kind == 6 && (i & 63) == 0) { a2 = make(-1074 + 53, -1000); c2 = make(-60, -20); }  // underflow edge
            const bool neg = rng() & 1;
            MulConst kc2 = make_const(c2), ks2 = make_const(s2);
            ok = (kc2.usable & ks2.usable) != 0;
            uint64_t d = dot2_rn(dbits(a2), kc2, dbits(b2), ks2, neg, ok);
            volatile double p1 = a2 * c2, p2 = b2 * s2;
            volatile double dref = neg ? p1 - p2 : p1 + p2;
            if (ok && d != dbits(dref)) {
                if (fails++ < 10)
                    std::printf("dot2 %a*%a %c %a*%a: got %a want %a\n", a2, c2, neg ? '-' : '+', b2, s2,
                                dfrom(d), (double)dref);
            }
            if (!ok) declined_dot++;
        }
    }
    // exact halfway quotients for divisors with an even significand:
    // x = y * (k + 1/2), so x / y rounds to the even neighbour of k + 1/2
    for (long i = 0; i < N / 20; i++) {
        const double ys[4] = {1.5, 1.25, 1.75, 1.125};
        const double yv = ys[i & 3];
        const uint64_t k = (rng() >> 17) | 1;                          // < 2^47: y * (k + 1/2) is exact
        const double xv = std::ldexp(yv * (double(k) + 0.5), int(rng() % 40) - 20);
        DivConst kd = make_div(yv);
        bool okh = true;
        const uint64_t q = div_fast(dbits(xv), kd, okh);
        volatile double qref = xv / yv;
        if (okh && q != dbits(qref)) {
            if (fails++ < 10) std::printf("div tie %a / %a: got %a want %a\n", xv, yv, dfrom(q), (double)qref);
        }
    }
    // the division by RN(sqrt(2)) on full random significands: the estimate
    // decides the rounding itself for all but about 2^-39 of them
    long declined_sqrt2 = 0;
    {
        const DivConst k2 = make_div(1.4142135623730951);
        for (long i = 0; i < N / 4; i++) {
            const double xv = dfrom((uint64_t(1023 - 40 + rng() % 44) << 52) | (rng() & MANT) |
                                    (rng() & 1 ? SIGN : 0));
            bool okq = true;
            const uint64_t q = div_fast(dbits(xv), k2, okq);
            volatile double qref = xv / 1.4142135623730951;
            if (!okq) declined_sqrt2++;
            else if (q != dbits(qref)) {
                if (fails++ < 10) std::printf("div_fast sqrt2 %a: got %a want %a\n", xv, dfrom(q), (double)qref);
            }
        }
    }
    {
        long declined_mid = 0;
        const long n_mid = near_midpoint_cases(1.4142135623730951, declined_mid, fails) +
                           near_midpoint_cases(1.0 + std::ldexp(1.0, -52) * 12345.0, declined_mid, fails);
        if (n_mid < 100 || declined_mid == 0) {
            std::printf("near-midpoint divisions: %ld cases, %ld declined\n", n_mid, declined_mid);
            return 5;
        }
    }
    if (declined_sqrt2 > 0) {
        std::printf("%ld declined divisions by sqrt(2)\n", declined_sqrt2);
        return 4;
    }
    // products that round up to a power of two (significand 2^53 before
    // normalisation), summed with a second product of the same exponent: two
    // such products of one sign make the largest sum the dot product forms
    long carry_cases = 0;
    for (long i = 0; i < N / 20; i++) {
        const double c3 = make(-6, 0), s3 = make(-6, 0);
        const int top_a = int(rng() & 1), top_b = int(rng() & 1);
        uint64_t ma, mb;
        if (!carry_significand(make_const(c3).m, top_a, ma)) continue;
        const bool both = (rng() % 4) != 0;
        if (both) {
            if (!carry_significand(make_const(s3).m, top_b, mb)) continue;
        } else {
            mb = (rng() & MANT) | HIDDEN;
        }
        const int ec = int((dbits(c3) >> 52) & 0x7FF) - 1023, es = int((dbits(s3) >> 52) & 0x7FF) - 1023;
        const int ea = int(rng() % 40) - 38;
        // RN(a*c) = 2^(ea+ec+1+top_a); RN(b*s) lands on the same exponent
        const int eb = ea + ec + top_a - es - (both ? top_b : 0);
        const double a3 = std::ldexp(double(ma), ea - 52) * ((rng() & 1) ? -1.0 : 1.0);
        const double b3 = std::ldexp(double(mb), eb - 52) * ((rng() & 1) ? -1.0 : 1.0);
        const bool neg = rng() & 1;
        MulConst kc3 = make_const(c3), ks3 = make_const(s3);
        bool okc = (kc3.usable & ks3.usable) != 0;
        const uint64_t d = dot2_rn(dbits(a3), kc3, dbits(b3), ks3, neg, okc);
        volatile double p1 = a3 * c3, p2 = b3 * s3;
        volatile double dref = neg ? p1 - p2 : p1 + p2;
        carry_cases++;
        if (okc && d != dbits(dref)) {
            if (fails++ < 10)
                std::printf("dot2 carry %a*%a %c %a*%a: got %a want %a\n", a3, c3, neg ? '-' : '+', b3, s3,
                            dfrom(d), (double)dref);
        }
    }
    if (carry_cases < N / 500) {
        std::printf("only %ld carry cases\n", carry_cases);
        return 3;
    }
    // the packed product of the mixed path, prod_pack: random and few-bit
    // significands, zeros of both signs, products that round up to a power
    // of two (with either position of the leading bit), and operands at and
    // beyond the edges of the normal range, which must decline or be exact
    long declined_pack = 0, pack_carry = 0;
    for (long i = 0; i < N; i++) {
        double c = (i & 15) == 0 ? make(-1022, 1023) : make(-6, 1);
        double a = (i & 15) == 1 ? make(-1022, 1023) : make(-80, 2);
        const int kind = int(rng() % 16);
        if (kind == 0) a = (rng() & 1) ? 0.0 : -0.0;
        if (kind == 1) {                                            // rounds up to 2^53
            uint64_t ma;
            const int top = int(rng() & 1);
            if (carry_significand(make_const(c).m, top, ma)) {
                a = std::ldexp(double(ma), int(rng() % 60) - 80) * ((rng() & 1) ? -1.0 : 1.0);
                pack_carry++;
            }
        }
        if (kind == 2) a = dfrom((rng() & MANT) | (rng() & 1 ? SIGN : 0));   // subnormal
        if (kind == 3) a = (rng() & 1) ? INFINITY : NAN;
        if (kind == 4) { a = make(1000, 1023); c = make(20, 1023); }           // overflow side
        if (kind == 5) { a = make(-1022, -1000); c = make(-60, -1); }           // underflow side
        if (kind == 6) c = make(-1022, -1000);
        const MulK k = make_mulk(c);
        bool ok = k.usable != 0;
        const uint64_t r = prod_pack(dbits(a), k, ok);
        volatile double ref = a * c;
        if (!ok) {
            if (k.usable && (kind <= 1 || kind >= 7)) declined_pack++;   // amplitude-like operands
            continue;
        }
        if (r != dbits(ref)) {
            if (fails++ < 10) std::printf("prod_pack %a * %a: got %a want %a\n", a, c, dfrom(r), (double)ref);
        }
        // a declined-free product must be normal or zero
        const int ef = int((r >> 52) & 0x7FF);
        if (!(ef != 0 && ef != 0x7FF) && (r & ~SIGN) != 0) {
            if (fails++ < 10) std::printf("prod_pack %a * %a accepted a non-normal result\n", a, c);
        }
    }
    {
        const double usable[4] = {1.0, -0.5, 0x1p-64, 1.9999999999999998};
        const double unusable[6] = {0.0, 2.0, 0x1.fffffffffffffp-65, 1e-300, INFINITY, 4.9e-324};
        for (double c : usable)
            if (!make_mulk(c).usable) { std::printf("constant %a should be usable\n", c); return 6; }
        for (double c : unusable)
            if (make_mulk(c).usable) { std::printf("constant %a should not be usable\n", c); return 6; }
    }
    if (pack_carry < N / 100) {
        std::printf("only %ld prod_pack carry cases\n", pack_carry);
        return 3;
    }
    if (declined_pack > N / 20) {
        std::printf("prod_pack declined %ld of %ld\n", declined_pack, N);
        return 2;
    }
    // every exponent field of a against a few constants: exact where
    // accepted, and accepted across the whole range a gate constant allows
    {
        const double cs[7] = {0.7071067811865476, -0.3826834323650898, 1.9999999999999998,
                              0.5, 2.2250738585072014e-300, 0x1p-64, -0x1.fffffffffffffp-65};
        for (double c : cs) {
            const MulK k = make_mulk(c);
            for (int ef = 0; ef <= 0x7FF; ef++) {
                for (int rep = 0; rep < 64; rep++) {
                    const double a = dfrom((uint64_t(ef) << 52) | (rng() & MANT) | (rep & 1 ? SIGN : 0));
                    bool ok = k.usable != 0;
                    const uint64_t r = prod_pack(dbits(a), k, ok);
                    volatile double ref = a * c;
                    const int rf = int((dbits(ref) >> 52) & 0x7FF);
                    if (ok && r != dbits(ref)) {
                        if (fails++ < 10)
                            std::printf("prod_pack edge %a * %a: got %a want %a\n", a, c, dfrom(r), (double)ref);
                    }
                    // a usable constant declines only operands whose exponent
                    // field lies outside [65, 2044] (zeros excepted)
                    (void)rf;
                    const bool zero_a = (dbits(a) & ~SIGN) == 0;
                    if (!ok && k.usable && !zero_a && ef >= 65 && ef <= 2044) {
                        if (fails++ < 10) std::printf("prod_pack declined %a * %a\n", a, c);
                    }
                    if (ok && !zero_a && (ef < 65 || ef > 2044)) {
                        if (fails++ < 10) std::printf("prod_pack accepted %a * %a\n", a, c);
                    }
                }
            }
        }
    }
    std::printf("cases %ld fails %ld declined mul %ld add %ld dot2 %ld prod_pack %ld (carries %ld)\n", N,
                fails, declined_mul, declined_add, declined_dot, declined_pack, pack_carry);
    if (fails) return 1;
    // declines must be rare on amplitude-like data
    if (declined_add > N / 100 || declined_dot > N / 50 || declined_div > N / 50) return 2;
    std::puts("dpemu ok");
    return 0;
}
