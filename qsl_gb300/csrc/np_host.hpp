// np_host.hpp -- host-side index arithmetic of the number-preserving layout.
//
// Plain C++ (no CUDA), so the CPU test suite compiles and checks it
// directly.  The compressed layout keeps the C(n, w) amplitudes of Hamming
// weight w in ascending order of their basis index: the order of qsl's
// generateLookup (src/utils/misc.cpp:75-90), which steps through them with
// Gosper's next-bit-permutation (misc.cpp:44-52).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>

namespace qslc {

constexpr int NPH_MAXN = 34;

// Pascal's triangle up to NPH_MAXN, built once on first use.
struct HostBinom {
    uint64_t v[NPH_MAXN + 1][NPH_MAXN + 1] = {};
    HostBinom()
    {
        for (int n = 0; n <= NPH_MAXN; n++) {
            v[n][0] = 1;
            for (int k = 1; k <= n; k++) v[n][k] = v[n - 1][k - 1] + (k <= n - 1 ? v[n - 1][k] : 0);
        }
    }
};

inline const HostBinom &host_binom()
{
    static const HostBinom b;
    return b;
}

inline uint64_t choose_u64(unsigned n, unsigned k)
{
    if (n > unsigned(NPH_MAXN) || k > n) return 0;
    return host_binom().v[n][k];
}

// Gosper's next integer with the same number of set bits (misc.cpp:44-52:
// t = x | (x-1); x = (t+1) | (((~t & -~t) - 1) >> (ctz(x)+1)), where -~t
// is t + 1).
inline uint64_t gosper_next(uint64_t x)
{
    const uint64_t t = x | (x - 1);
    return (t + 1) | (((~t & (t + 1)) - 1) >> (__builtin_ctzll(x) + 1));
}

// Slot of basis index y among the weight-popcount(y) integers: the sum over
// its set bits, the i-th lowest at position p_i, of C(p_i, i).
inline uint64_t rank_of(uint64_t y)
{
    uint64_t r = 0;
    unsigned i = 0;
    for (unsigned p = 0; y != 0 && p <= unsigned(NPH_MAXN); p++, y >>= 1)
        if (y & 1) r += choose_u64(p, ++i);
    return r;
}

// Basis index of slot r among the w-weight integers of n bits.
inline uint64_t unrank_of(uint64_t r, unsigned n, unsigned w)
{
    uint64_t x = 0;
    for (int p = int(n) - 1; p >= 0 && w > 0; p--) {
        const uint64_t c = choose_u64(unsigned(p), w);
        if (c <= r) {
            x |= uint64_t(1) << p;
            r -= c;
            w--;
        }
    }
    return x;
}

// compressed -> full 2^n vector (zeros outside the sector); `ab` bytes per
// amplitude.
inline void np_scatter(const void *comp, void *full, unsigned n, unsigned w, size_t ab)
{
    const auto *c = static_cast<const unsigned char *>(comp);
    auto *f = static_cast<unsigned char *>(full);
    std::memset(f, 0, (size_t(1) << n) * ab);
    const uint64_t cnt = choose_u64(n, w);
    uint64_t x = (uint64_t(1) << w) - 1;
    for (uint64_t r = 0; r < cnt; r++) {
        std::memcpy(f + x * ab, c + r * ab, ab);
        if (r + 1 < cnt) x = gosper_next(x);
    }
}

// full 2^n vector -> compressed (the weight-w amplitudes, ascending)
inline void np_gather(const void *full, void *comp, unsigned n, unsigned w, size_t ab)
{
    const auto *f = static_cast<const unsigned char *>(full);
    auto *c = static_cast<unsigned char *>(comp);
    const uint64_t cnt = choose_u64(n, w);
    uint64_t x = (uint64_t(1) << w) - 1;
    for (uint64_t r = 0; r < cnt; r++) {
        std::memcpy(c + r * ab, f + x * ab, ab);
        if (r + 1 < cnt) x = gosper_next(x);
    }
}

}  // namespace qslc
