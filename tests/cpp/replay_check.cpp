// Checks the exact sequential-sum replay (qsl_gb300/csrc/replay.cuh) on the
// CPU: for random runs of terms, composing per-term transducers in binade e
// and adding the grid steps to a start sum gives exactly the sequential
// rounded sum, whenever the sum stays in the binade -- with ties (float
// terms in a double sum, equal terms) and without; and the composition is
// associative (any grouping gives the same counts).
#include "replay.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
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

// grid_ceil(u, e) is the first grid position of binade e at or above u.
static int check_ceil(int trials)
{
    int fails = 0;
    for (int t = 0; t < trials; t++) {
        const int e = -int(rng() % 60);
        double u = std::ldexp(double(rng() >> 11) * 0x1p-53, -int(rng() % 70));
        if (rng() % 8 == 0) u = std::ldexp(double(rng() % 1000), e - 52);   // on the grid
        if (rng() % 16 == 0) u = 0;
        const uint64_t n = grid_ceil<double>(u, e);
        if (n >= (uint64_t(1) << 53)) continue;
        const bool ok = (n == 0 && u == 0) ||
                        (n > 0 && std::ldexp(double(n - 1), e - 52) < u && u <= std::ldexp(double(n), e - 52));
        if (!ok && fails++ < 5) std::printf("grid_ceil(%a, %d) = %llu\n", u, e, (unsigned long long)n);
    }
    std::printf("grid_ceil: %d fails\n", fails);
    return fails;
}

static uint64_t bits_of(double x)
{
    uint64_t b;
    std::memcpy(&b, &x, 8);
    return b;
}

// The reference's merge: the sequential running sum against sorted uniforms.
static std::vector<uint64_t> cdf_sequential(const std::vector<double> &p, const std::vector<double> &u)
{
    std::vector<uint64_t> out(u.size(), 0);
    size_t k = 0;
    double run = 0;
    for (size_t i = 0; i < p.size() && k < u.size(); i++) {
        volatile double nx = run + p[i];
        run = nx;
        while (k < u.size() && u[k] <= run) out[k++] = i;
    }
    return out;
}

// The batching form's warp walk (warp_walk in batch.cu), its 32 lanes
// emulated one after another: rounds of 32 runs of `run` terms in one
// binade, a scan of the runs' transducers, the walks, the first term that
// leaves the binade added on its own; zero sums skip zero terms 32 at a
// time, subnormal sums add one term at a time.  A is the sum's type (the
// terms are doubles); with uniforms, the sum is a CDF and each uniform's
// outcome goes to `out`.
template <class A>
static A add_term(A s, double t)
{
    volatile A r = s + A(t);
    return r;
}

template <class A>
static A walk_rounds(const std::vector<double> &p, const std::vector<double> *u, std::vector<uint64_t> *out,
                     unsigned run)
{
    const uint64_t dim = p.size(), NONE = ~uint64_t(0);
    const size_t ns = u ? u->size() : 0;
    size_t k = 0;
    A s = 0;
    uint64_t i = 0;
    auto consume = [&](uint64_t idx) {
        while (k < ns && bits_of((*u)[k]) <= bits_of(double(s))) (*out)[k++] = idx;
    };
    while (i < dim && (!u || k < ns)) {
        const int e = binade<A>(s);
        if (e < fp_traits<A>::EMIN) {
            if (to_bits(s) == 0) {
                unsigned first = 32;
                for (unsigned l = 0; l < 32; l++)
                    if (i + l < dim && bits_of(p[i + l]) != 0) {
                        first = l;
                        break;
                    }
                consume(i);
                if (first == 32) {
                    i = i + 32 < dim ? i + 32 : dim;
                    continue;
                }
                i += first;
            }
            s = add_term(s, p[i]);
            consume(i);
            i++;
            continue;
        }
        const uint64_t m0 = grid_pos(s);
        const uint64_t end = i + 32 * run < dim ? i + 32 * run : dim;
        uint64_t base[32], pos0[32], pos[32];
        unsigned len[32];
        Tx acc = tx_identity();
        uint64_t bad = NONE;
        for (unsigned l = 0; l < 32; l++) {
            base[l] = i + uint64_t(l) * run;
            len[l] = base[l] < end ? unsigned(end - base[l] < run ? end - base[l] : run) : 0u;
            const double *pl = p.data() + base[l];
            auto get = [pl](unsigned r) { return pl[r]; };
            bool big = false;
            const Tx t = run_effect<A>(get, len[l], e, big);
            pos0[l] = m0 + acc.d[m0 & 1];
            acc = tx_then(acc, t);
            pos[l] = pos0[l];
            const unsigned walked = run_walk<A>(get, len[l], e, pos[l]);
            if (walked < len[l] && base[l] + walked < bad) bad = base[l] + walked;
        }
        const uint64_t stop = bad == NONE ? end : bad;
        const uint64_t last = bad == NONE ? end - 1 : stop;
        const uint64_t pend = pos[(last - i) / run];
        while (k < ns) {
            const uint64_t tgt = grid_ceil<A>(A((*u)[k]), e);
            if (tgt > pend) break;
            unsigned L = 32;
            for (unsigned l = 0; l < 32; l++)
                if (len[l] && base[l] < stop && pos[l] >= tgt) {
                    L = l;
                    break;
                }
            if (L == 32) break;
            const double *pL = p.data() + base[L];
            (*out)[k++] = base[L] + run_find<A>([pL](unsigned r) { return pL[r]; }, len[L], e, pos0[L], tgt);
        }
        s = grid_at<A>(pend, e);
        i = stop;
        if (bad != NONE) {
            s = add_term(s, p[i]);
            consume(i);
            i++;
        }
    }
    return s;
}

static std::vector<uint64_t> cdf_rounds(const std::vector<double> &p, const std::vector<double> &u,
                                        unsigned run)
{
    std::vector<uint64_t> out(u.size(), 0);
    walk_rounds<double>(p, &u, &out, run);
    return out;
}

// Probability-like sums: the walk's total against the sequential sum, in
// double, and in float over float terms (held as doubles).
static int check_sums(int trials)
{
    int fails = 0, cases = 0;
    for (int t = 0; t < trials; t++) {
        const uint64_t dim = 1 + rng() % 20000;
        std::vector<double> p(dim);
        std::normal_distribution<double> g;
        const int kind = int(rng() % 4);
        for (auto &x : p) {
            const double re = g(rng), im = g(rng);
            x = std::ldexp(re * re + im * im, -int(rng() % 3) - 14);
            if (kind == 1 && rng() % 3 == 0) x = 0;
            if (kind == 2) x = std::ldexp(1.0, -14);
            if (kind == 3) x = std::ldexp(double(rng() % 5), -149);        // float subnormals
        }
        double sd = 0;
        for (double x : p) sd = add_term(sd, x);
        std::vector<double> pf(p.begin(), p.end());
        for (auto &x : pf) x = double(float(x));
        float sf = 0;
        for (double x : pf) sf = add_term(sf, x);
        for (unsigned r : {1u, 16u}) {
            cases += 2;
            const double gd = walk_rounds<double>(p, nullptr, nullptr, r);
            const float gf = walk_rounds<float>(pf, nullptr, nullptr, r);
            if (bits_of(gd) != bits_of(sd) && fails++ < 5) std::printf("double sum differs: kind %d\n", kind);
            if (to_bits(gf) != to_bits(sf) && fails++ < 5) std::printf("float sum differs: kind %d\n", kind);
        }
    }
    std::printf("sums: %d cases, %d fails\n", cases, fails);
    return fails;
}

// Term sequences that exercise every path of the walk: |a|^2 of random
// states, leading zeros, equal dyadic terms (exact sums), terms from a few
// dyadic values (ties), subnormal terms, and a term far above the sum.
static int check_cdf_walk(int trials)
{
    int fails = 0, cases = 0;
    for (int t = 0; t < trials; t++) {
        const int n = 3 + int(rng() % 12);
        const uint64_t dim = uint64_t(1) << n;
        std::vector<double> p(dim);
        const int kind = int(rng() % 7);
        std::normal_distribution<double> g;
        double norm = 0;
        for (auto &x : p) {
            const double re = g(rng), im = g(rng);
            x = re * re + im * im;
            norm += x;
        }
        for (auto &x : p) x /= norm;
        if (kind == 1)
            for (uint64_t j = 0; j < dim / 2 + rng() % (dim / 2); j++) p[j] = 0;
        if (kind == 2)
            for (auto &x : p) x = std::ldexp(1.0, -n);
        if (kind == 3) {
            const double vals[4] = {0x1p-20, 0x1.8p-30, 0x1.0000000000001p-12, 0x1p-55};
            for (auto &x : p) x = vals[rng() % 4];
        }
        if (kind == 4)
            for (uint64_t j = 0; j < dim; j++) p[j] = j < dim / 2 ? std::ldexp(double(rng() % 7), -1074) : p[j];
        if (kind == 5) p[rng() % dim] = 0.75;
        if (kind == 6)
            for (auto &x : p) x = double(float(x));
        std::vector<double> cdf(dim);
        double run = 0;
        for (uint64_t j = 0; j < dim; j++) {
            volatile double nx = run + p[j];
            run = nx;
            cdf[j] = run;
        }
        std::vector<double> u;
        for (int j = 0; j < 64; j++) u.push_back(double(rng() >> 11) * 0x1p-53);
        for (int j = 0; j < 16; j++) u.push_back(cdf[rng() % dim]);                 // on a partial sum
        for (int j = 0; j < 8; j++) u.push_back(std::nextafter(cdf[rng() % dim], 1.0));
        u.push_back(0.0);
        u.push_back(std::nextafter(run, 2.0));                                       // above the total
        std::sort(u.begin(), u.end());
        const auto want = cdf_sequential(p, u);
        for (unsigned r : {1u, 3u, 16u}) {
            cases++;
            if (cdf_rounds(p, u, r) != want && fails++ < 5)
                std::printf("cdf walk differs: kind %d, n %d, run %u\n", kind, n, r);
        }
    }
    std::printf("cdf walk: %d cases, %d fails\n", cases, fails);
    return fails;
}

int main()
{
    int f = check<double, double>(3000) + check<double, float>(3000) + check<float, float>(3000);
    f += check_ceil(200000);
    f += check_cdf_walk(1500);
    f += check_sums(600);
    if (f) return 1;
    std::puts("replay ok");
    return 0;
}
