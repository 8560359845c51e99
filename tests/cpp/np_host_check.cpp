// Checks the host-side index arithmetic of the number-preserving layout
// (qsl_gb300/csrc/np_host.hpp) against brute force: Gosper stepping equals
// the ascending list of fixed-weight integers (the order of qsl's
// generateLookup, src/utils/misc.cpp:75-90), rank/unrank are inverse and
// equal the position in that list, scatter/gather round-trip.
#include "np_host.hpp"

#include <cstdio>
#include <vector>

using namespace qslc;

static int fails = 0;
#define CHECK(c)                                                       \
    do {                                                               \
        if (!(c)) {                                                    \
            std::fprintf(stderr, "FAIL %s:%d %s\n", __FILE__, __LINE__, #c); \
            if (++fails > 20) return 1;                                \
        }                                                              \
    } while (0)

int main()
{
    for (unsigned n = 1; n <= 16; n++) {
        for (unsigned w = 0; w <= n; w++) {
            std::vector<uint64_t> ref;
            for (uint64_t y = 0; y < (uint64_t(1) << n); y++)
                if (unsigned(__builtin_popcountll(y)) == w) ref.push_back(y);
            CHECK(ref.size() == choose_u64(n, w));
            uint64_t x = (uint64_t(1) << w) - 1;
            for (size_t i = 0; i < ref.size(); i++) {
                CHECK(x == ref[i]);
                CHECK(rank_of(ref[i]) == i);
                CHECK(unrank_of(i, n, w) == ref[i]);
                if (w > 0 && i + 1 < ref.size()) x = gosper_next(x);
            }
            if (w == 0 || w == n) continue;
            std::vector<double> full((size_t(2) << n), 0.0), back((size_t(2) << n), -1.0);
            std::vector<double> comp(2 * ref.size());
            for (size_t i = 0; i < ref.size(); i++) {
                full[2 * ref[i]] = double(i) + 0.25;
                full[2 * ref[i] + 1] = -double(i);
            }
            np_gather(full.data(), comp.data(), n, w, 16);
            for (size_t i = 0; i < ref.size(); i++) CHECK(comp[2 * i] == double(i) + 0.25);
            np_scatter(comp.data(), back.data(), n, w, 16);
            CHECK(back == full);
        }
    }
    // spot checks at 28..32 qubits against the combinatorial definition
    for (unsigned n : {28u, 30u, 32u}) {
        unsigned w = n / 2;
        uint64_t cnt = choose_u64(n, w);
        for (uint64_t r : {uint64_t(0), uint64_t(1), cnt / 3, cnt / 2, cnt - 2, cnt - 1}) {
            uint64_t y = unrank_of(r, n, w);
            CHECK(unsigned(__builtin_popcountll(y)) == w && y < (uint64_t(1) << n));
            CHECK(rank_of(y) == r);
            if (r + 1 < cnt) CHECK(gosper_next(y) == unrank_of(r + 1, n, w));
        }
    }
    CHECK(choose_u64(28, 14) == 40116600ull);
    if (fails) return 1;
    std::puts("np_host ok");
    return 0;
}
