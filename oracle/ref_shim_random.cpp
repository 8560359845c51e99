// ref_shim_random.cpp -- seedable stand-in for qsl's src/utils/random.cpp.
//
// TEST INFRASTRUCTURE ONLY: linked into oracle/_ref/libqslref.so together
// with the reference's own, unmodified sources so that the reference can be
// run deterministically.  The reference seeds std::mt19937 from
// std::random_device (src/utils/random.cpp:33-40) and has no seed hook; this
// file defines the same members (include/qsl/utils/random.hpp:51-78) with
// two additions:
//   * every new Random object draws its seed from a global, settable
//     sequence (qslref_seed);
//   * getNum() can be fed an explicit list of uniforms
//     (qslref_set_uniforms), which it hands out in order before falling
//     back to the generator.  This is how the same uniforms reach the
//     reference, the restatement and the CUDA backend.
#include <cstddef>
#include <cstdint>
#include <random>
#include <vector>

#include "qsl/utils/random.hpp"
#include "qsl/utils/quantum.hpp"
#include "qsl/utils/misc.hpp"

namespace {
std::uint32_t g_next_seed = 5489u;
std::vector<double> g_feed;
std::size_t g_feed_pos = 0;
}  // namespace

extern "C" void qslref_seed(std::uint32_t seed) { g_next_seed = seed; }

extern "C" void qslref_set_uniforms(const double *u, std::size_t n)
{
    g_feed.assign(u, u + n);
    g_feed_pos = 0;
}

extern "C" std::size_t qslref_uniforms_left(void)
{
    return g_feed.size() - g_feed_pos;
}

namespace qsl {

template <std::floating_point Fp>
Random<Fp>::Random(Fp a, Fp b)
{
    generator = std::mt19937(g_next_seed++);
    distribution = std::uniform_real_distribution<Fp>(a, b);
}

template <std::floating_point Fp>
Fp Random<Fp>::getNum()
{
    if (g_feed_pos < g_feed.size()) return static_cast<Fp>(g_feed[g_feed_pos++]);
    return distribution(generator);
}

// The state generators keep the reference's behaviour (uniform [-1, 1)
// real and imaginary parts, normalised) on the seeded generator.
template <std::floating_point Fp>
std::vector<complex<Fp>> makeRandomState(unsigned nqubits)
{
    std::size_t dim = std::size_t(1) << nqubits;
    Random<Fp> random(-1, 1);
    std::vector<complex<Fp>> state;
    for (std::size_t i = 0; i < dim; i++) {
        Fp re = random.getNum();
        Fp im = random.getNum();
        state.push_back(complex<Fp>(re, im));
    }
    normalise(state);
    return state;
}

template <std::floating_point Fp>
std::vector<complex<Fp>> makeRandomNPState(unsigned nqubits, unsigned nones)
{
    Random<Fp> random{-1, 1};
    std::size_t dim = std::size_t(1) << nqubits;
    std::size_t x = (1ULL << nones) - 1;
    std::size_t end = x << (nqubits - nones);
    std::vector<complex<Fp>> state(dim);
    while (x <= end) {
        Fp re = random.getNum();
        Fp im = random.getNum();
        state[x] = complex<Fp>(re, im);
        next(x);
    }
    normalise(state);
    return state;
}

template <std::floating_point Fp>
std::vector<complex<Fp>> makeRandomNPState(unsigned nqubits)
{
    std::mt19937 gen{g_next_seed++};
    std::uniform_int_distribution<unsigned> dist(1, nqubits - 1);
    return makeRandomNPState<Fp>(nqubits, dist(gen));
}

template <std::floating_point Fp>
std::vector<Fp> makeRandomPhases(int test_len)
{
    std::vector<Fp> out;
    Random<Fp> random(-M_PI, M_PI);
    for (int i = 0; i < test_len; i++) out.push_back(random.getNum());
    return out;
}

template class Random<float>;
template class Random<double>;
template std::vector<complex<float>> makeRandomState(unsigned);
template std::vector<complex<double>> makeRandomState(unsigned);
template std::vector<complex<float>> makeRandomNPState(unsigned);
template std::vector<complex<double>> makeRandomNPState(unsigned);
template std::vector<complex<float>> makeRandomNPState(unsigned, unsigned);
template std::vector<complex<double>> makeRandomNPState(unsigned, unsigned);
template std::vector<float> makeRandomPhases(int);
template std::vector<double> makeRandomPhases(int);

}  // namespace qsl
