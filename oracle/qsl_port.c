/*
 * qsl_port.c -- the oracle: a plain-C restatement of qsl's CPU algorithms
 * for the state-vector hot path (Default / OpenMP / NP backends).
 *
 * TEST INFRASTRUCTURE ONLY.  The parity tests, the smoke check and the
 * CPU-baseline leg of the benchmark load this library as the checker; the
 * CUDA backend never links or calls it.
 *
 * Pinned against the reference itself: tests/golden/ holds outputs of the
 * reference library (src/qubits, src/utils compiled unmodified, with a
 * seedable replacement for src/utils/random.cpp) that the tests compare
 * this restatement with.
 *
 * Build: gcc -O2 -ffp-contract=off -fopenmp -fPIC -shared (see Makefile).
 * -ffp-contract=off keeps every a*b+c as a rounded product and a rounded
 * sum, as the reference's x86-64 build computes it.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "qsl_port.h"

#ifdef _OPENMP
/* The reference's Omp backend parallelises the outermost loop of each
 * sweep with a static schedule (src/qubits/omp/gates.cpp:166-200). */
#define OMP_FOR(nth) _Pragma("omp parallel for schedule(static) num_threads(nth) if(nth > 1)")
#else
#define OMP_FOR(nth)
#endif

#define FP double
#define SFX d
#define COS cos
#define SIN sin
#define SQRT sqrt
#include "port_body.inc"
#undef FP
#undef SFX
#undef COS
#undef SIN
#undef SQRT

#define FP float
#define SFX f
#define COS cosf
#define SIN sinf
#define SQRT sqrtf
#include "port_body.inc"
#undef FP
#undef SFX
#undef COS
#undef SIN
#undef SQRT

/* ------------------------------------------------------------------ */
/* Bit utilities: src/utils/misc.cpp                                   */
/* ------------------------------------------------------------------ */

/* misc.cpp:44-52: Gosper's next bit permutation.  The reference's ctz is
 * the 32-bit __builtin_ctz (misc.cpp:36), so only the low 32 bits of x
 * take part in it, as here. */
uint64_t port_next(uint64_t x)
{
    uint64_t t = x | (x - 1);
    unsigned low = (unsigned)x;
    unsigned tz = low ? (unsigned)__builtin_ctz(low) : 32u;
    return (t + 1) | (((~t & -~t) - 1) >> (tz + 1));
}

/* misc.cpp:54-62 */
unsigned port_hamming_weight(uint64_t n)
{
    unsigned c = 0;
    while (n) { c += (unsigned)(n & 1); n >>= 1; }
    return c;
}

/* misc.cpp:65-73 (unsigned arithmetic, wraps as the reference does) */
unsigned port_choose(unsigned n, unsigned k)
{
    unsigned ans = 1;
    for (unsigned i = 1; i <= k; i++) { ans *= (n - k + i); ans /= i; }
    return ans;
}

/* misc.cpp:75-90: ascending integers of `ones` set bits in `len` bits.
 * Writes up to `cap` entries into `out` (out may be NULL to count) and
 * returns the table length.  ones > len has no entries. */
size_t port_generate_lookup(unsigned len, unsigned ones, uint64_t *out,
                            size_t cap)
{
    if (ones > len || len > 63) return 0;
    uint64_t x = (ones == 64) ? ~0ull : ((1ull << ones) - 1ull);
    uint64_t end = x << (len - ones);
    size_t m = 0;
    while (x <= end) {
        if (out && m < cap) out[m] = x;
        m++;
        if (ones == 0) break;          /* {0} is the only entry */
        x = port_next(x);
    }
    return m;
}

/* quantum.cpp:133-156: weight of the nonzero amplitudes; -1 when two
 * nonzero amplitudes have different weights (the reference throws). */
int port_check_state_np_d(const double *s, unsigned n)
{
    size_t dim = (size_t)1 << n;
    int w = 0, found = 0;
    for (size_t i = 0; i < dim; i++) {
        double a = s[2 * i] * s[2 * i] + s[2 * i + 1] * s[2 * i + 1];
        if (a != 0) {
            int hw = (int)port_hamming_weight(i);
            if (!found) { w = hw; found = 1; }
            else if (w != hw) return -1;
        }
    }
    return w;
}

int port_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
