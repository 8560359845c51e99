// Checks the exact sequential-sum replay (qsl_gb300/csrc/replay.cuh) on the
// CPU: for random runs of terms, composing per-term transducers in binade e
// and adding the grid steps to a start sum gives exactly the sequential
// rounded sum, whenever the sum stays in the binade -- with ties (float
// terms in a double sum, equal terms) and without; and the composition is
// associative (any grouping gives the same counts).
#include "replay.cuh"

#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

using namespace qslc;
static std::mt19937_64 rng(99);

template <class A, class P>
static int check(int trials)
{
    using T = fp_traits<A>;
    int fails = 0, valid = 0;
    for (int t = 0; t < trials; t++) {
        const int len = 1 + int(rng() % 3000);
        const int scale = -int(rng() % 40) - 1;
        std::vector<P> p(len);
        for (auto &x : p) {
            double v = std::ldexp(double(rng() >> 11) * 0x1p-53, scale);
            if (rng() % 4 == 0) v = std::ldexp(1.0, scale);            // many equal terms: ties
            if (rng() % 16 == 0) v = 0;
            x = P(v);
        }
        A s = A(std::ldexp(1.0 + double(rng() >> 11) * 0x1p-53, scale + 8));
        if (rng() % 2) s = A(std::ldexp(1.0, scale + 10));
        const int e = binade<A>(s);
        // sequential
        A seq = s;
        bool stays = true;
        for (P x : p) {
            volatile A nx = seq + A(x);
            seq = nx;
            if (binade<A>(seq) != e) stays = false;
        }
        // transducers, grouped two ways
        Tx all = tx_identity(), left = tx_identity(), right = tx_identity();
        bool big_any = false;
        for (int i = 0; i < len; i++) {
            bool tie, big;
            uint64_t q = grid_steps<A>(A(p[i]), e, tie, big);
            big_any |= big;
            const Tx term = tx_term(q, tie);
            all = tx_then(all, term);
            if (i < len / 2) left = tx_then(left, term);
            else right = tx_then(right, term);
        }
        const Tx grouped = tx_then(left, right);
        if (grouped.d[0] != all.d[0] || grouped.d[1] != all.d[1]) fails++;
        const uint64_t s0 = uint64_t(std::ldexp(double(s), T::MANT - e));
        const uint64_t d = all.d[s0 & 1];
        if (!stays || big_any || s0 + d >= (uint64_t(1) << (T::MANT + 1))) continue;
        valid++;
        const A got = A(std::ldexp(double(s0 + d), e - T::MANT));
        if (got != seq) {
            if (fails++ < 5) std::printf("mismatch len %d: %a vs %a\n", len, double(got), double(seq));
        }
    }
    std::printf("%s/%s: %d valid runs checked, %d fails\n", sizeof(A) == 8 ? "double" : "float",
                sizeof(P) == 8 ? "double" : "float", valid, fails);
    return fails;
}

int main()
{
    int f = check<double, double>(3000) + check<double, float>(3000) + check<float, float>(3000);
    if (f) return 1;
    std::puts("replay ok");
    return 0;
}
