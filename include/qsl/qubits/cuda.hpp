/*
 * qsl/qubits/cuda.hpp -- qsl::Qubits on one GB300 GPU.
 *
 *   qsl::Qubits<qsl::Type::Cuda, Fp>        drop-in for Type::Default / Type::Omp
 *   qsl::Qubits<qsl::Type::CudaNP, Fp>      drop-in for Type::NP / Type::OmpNP
 *   qsl::Qubits<qsl::Type::CudaResize, Fp>  drop-in for Type::Resize
 *
 * They keep the member signatures of include/qsl/qubits/default.hpp:97-712,
 * np.hpp:100-250 and resize.hpp:46-370 of qsl, so qsl's templated consumers (the Simulator /
 * HasAllGates / HasMeasurement / NPSimulator concepts of concepts.hpp, the
 * Verify checkers, the benchmark Time/Compare templates) instantiate with
 * them unchanged.  Every call goes through the C ABI of include/qslc.h to the
 * CUDA kernels in libqslc.so; the amplitudes live in device memory.
 *
 * Use with qsl's headers: include <qsl/qubits.hpp> first.  qsl's Type enum
 * has no Cuda enumerator; qsl::cuda_type / qsl::cuda_np_type /
 * qsl::cuda_resize_type name the three backends (they equal Type::Cuda /
 * Type::CudaNP / Type::CudaResize once those enumerators are added with the
 * values 0x100 / 0x101 / 0x102).  Without qsl's headers, this file pulls in
 * qsl/cuda_standalone.hpp, whose Type enum has all three.
 *
 * Errors: std::logic_error where qsl throws it (size mismatch, mixed
 * Hamming weight, bad number of ones) and for out-of-range qubit indices
 * (undefined behaviour in qsl); std::runtime_error for CUDA failures.
 *
 * Random numbers: each object owns a std::mt19937 with
 * std::uniform_real_distribution<Fp>(0, 1), seeded from std::random_device
 * like qsl::Random (src/utils/random.cpp:33-45); seed() fixes it.  The
 * resizeable backend shares one generator per Fp among all its objects, as
 * qsl's Resize backend does (its `random` is a static member,
 * resize.hpp:59).  The uniforms are drawn on the host in the reference's
 * order and passed to the device, so a given seed gives the reference's
 * outcomes.
 */
#ifndef QSL_QUBITS_CUDA_HPP
#define QSL_QUBITS_CUDA_HPP

#if defined(QSL_QUBITS_HPP)
/* qsl's own declarations are in scope */
#elif defined(QSL_COMPLEX_HPP)
#error "include <qsl/qubits.hpp> before <qsl/qubits/cuda.hpp>"
#else
#include "../cuda_standalone.hpp"
#endif

#include <cstddef>
#include <cstdint>
#include <iostream>
#include <map>
#include <random>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "../../qslc.h"

namespace qsl {

inline constexpr Type cuda_type = static_cast<Type>(0x100);
inline constexpr Type cuda_np_type = static_cast<Type>(0x101);
inline constexpr Type cuda_resize_type = static_cast<Type>(0x102);

namespace cuda_detail {

inline void check(int rc)
{
    if (rc == QSLC_OK) return;
    std::string msg = qslc_last_error();
    if (rc == QSLC_EINVAL || rc == QSLC_ESIZE || rc == QSLC_ENOTNP) throw std::logic_error(msg);
    throw std::runtime_error(msg);
}

template <class Fp>
inline constexpr int dtype_of = std::is_same_v<Fp, double> ? QSLC_C128 : QSLC_C64;

// checkStateSize (src/utils/quantum.cpp:108-131)
inline unsigned log2_size(std::size_t n)
{
    if (n == 0 || (n & (n - 1)) != 0) throw std::logic_error("State vector size is not a power of two");
    unsigned len = 0;
    while (n > 1) { n >>= 1; len++; }
    return len;
}

/* State handling, measurement and randomness shared by both backends. */
template <std::floating_point Fp>
class Base {
protected:
    qslc_state *h = nullptr;
    std::mt19937 generator;
    std::uniform_real_distribution<Fp> distribution{Fp(0), Fp(1)};
    bool shared_rng = false;   // draw from the one generator of all such objects

    struct Shared {
        std::mt19937 generator{std::random_device{}()};
        std::uniform_real_distribution<Fp> distribution{Fp(0), Fp(1)};
    };
    static Shared &shared()
    {
        static Shared s;
        return s;
    }

    Base() : generator(std::random_device{}()) {}
    Base(const Base &o)
        : generator(o.generator), distribution(o.distribution), shared_rng(o.shared_rng)
    {
        check(qslc_clone(o.h, &h));
    }
    Base(Base &&o) noexcept
        : h(o.h), generator(o.generator), distribution(o.distribution), shared_rng(o.shared_rng)
    {
        o.h = nullptr;
    }
    ~Base()
    {
        if (h) qslc_destroy(h);
    }
    void assign(const Base &o) { check(qslc_assign(h, o.h)); }
    Fp draw()
    {
        if (shared_rng) return shared().distribution(shared().generator);
        return distribution(generator);
    }
    void gate1(int g, unsigned t, Fp a = 0) { check(qslc_gate1(h, g, t, double(a))); }
    void gate2(int g, unsigned a, unsigned b, Fp x = 0) { check(qslc_gate2(h, g, a, b, double(x))); }

public:
    using Fp_type = Fp;

    /// Fix the generator's seed (qsl::Random has no equivalent).
    void seed(std::uint32_t s)
    {
        if (shared_rng) {
            shared().generator.seed(s);
            shared().distribution.reset();
        } else {
            generator.seed(s);
            distribution.reset();
        }
    }
    /// The C-ABI handle, for callers that mix in qslc_* calls.
    qslc_state *handle() const { return h; }
    /// Wait for every queued kernel of this object.
    void synchronize() const { check(qslc_synchronize(h)); }

    unsigned getNumQubits() const { return qslc_num_qubits(h); }

    void reset() { check(qslc_reset(h)); }

    std::vector<complex<Fp>> getState() const
    {
        std::vector<complex<Fp>> out(std::size_t(1) << getNumQubits());
        check(qslc_get_state(h, out.data(), out.size()));
        return out;
    }

    void setState(const std::vector<complex<Fp>> &state)
    {
        check(qslc_set_state(h, state.data(), state.size()));
    }

    void setBasisState(std::size_t index) { check(qslc_set_basis(h, index)); }

    void print(std::ostream &os = std::cout) const
    {
        os << "Number of qubits = " << getNumQubits() << std::endl;
        for (const auto &a : getState()) os << "(" << a.real << ", " << a.imag << ")" << std::endl;
        os << std::endl;
    }

    // Measurement (src/qubits/default/measure.cpp) ---------------------
    Fp prob(unsigned targ, unsigned outcome) const
    {
        double p = 0;
        check(qslc_prob(h, targ, outcome, &p));
        return Fp(p);
    }

    int measure(unsigned targ)
    {
        const Fp u = draw();
        int out = 0;
        check(qslc_measure(h, targ, double(u), &out));
        return out;
    }

    std::size_t measureAll()
    {
        const Fp u = draw();
        std::uint64_t out = 0;
        check(qslc_measure_all(h, double(u), &out));
        return std::size_t(out);
    }

    Fp postselect(unsigned targ, unsigned outcome)
    {
        double p = 0;
        check(qslc_postselect(h, targ, outcome, &p));
        return Fp(p);
    }

    std::vector<std::size_t> sample(unsigned targ, std::size_t nsamples)
    {
        std::vector<double> u(nsamples);
        for (auto &x : u) x = double(draw());
        std::uint64_t c[2] = {0, 0};
        check(qslc_sample(h, targ, u.data(), u.size(), c));
        return {std::size_t(c[0]), std::size_t(c[1])};
    }

    std::map<std::size_t, std::size_t> sampleAll(std::size_t nsamples)
    {
        std::vector<double> u(nsamples);
        for (auto &x : u) x = double(draw());
        std::vector<std::uint64_t> shots(nsamples);
        check(qslc_sample_all(h, u.data(), u.size(), shots.data()));
        std::map<std::size_t, std::size_t> results;
        for (auto s : shots) results[std::size_t(s)]++;
        return results;
    }

    /// sampleAll2 (measure.cpp:237-267): every basis index is a key of the
    /// result (np/measure.cpp:259-289: every index of the preserved weight).
    std::map<std::size_t, std::size_t> sampleAll2(std::size_t nsamples)
    {
        std::vector<double> u(nsamples);
        for (auto &x : u) x = double(draw());
        std::vector<std::uint64_t> bins(nsamples);
        check(qslc_sample_all2(h, u.data(), u.size(), bins.data()));
        std::map<std::size_t, std::size_t> results;
        const unsigned n = getNumQubits();
        if (qslc_is_np(h)) {
            unsigned w = 0;
            check(qslc_num_ones(h, &w));
            std::uint64_t x = (std::uint64_t(1) << w) - 1;
            const std::uint64_t end = x << (n - w);
            while (true) {
                results[std::size_t(x)] = 0;
                if (x == end) break;
                const std::uint64_t t = x | (x - 1);
                x = (t + 1) | (((~t & (t + 1)) - 1) >> (__builtin_ctzll(x) + 1));
            }
        } else {
            for (std::size_t i = 0; i < (std::size_t(1) << n); i++) results[i] = 0;
        }
        for (auto b : bins)
            if (b != ~std::uint64_t(0)) results[std::size_t(b)]++;
        return results;
    }

    // Gates every backend has (HasNPGates, concepts.hpp:65-82) ---------
    void pauliZ(unsigned targ) { gate1(QSLC_PAULI_Z, targ); }
    void rotateZ(unsigned targ, Fp angle) { gate1(QSLC_ROTATE_Z, targ, angle); }
    void phase(unsigned targ, Fp angle) { gate1(QSLC_PHASE, targ, angle); }
    void controlZ(unsigned ctrl, unsigned targ) { gate2(QSLC_CONTROL_Z, ctrl, targ); }
    void controlRotateZ(unsigned ctrl, unsigned targ, Fp angle)
    {
        gate2(QSLC_CONTROL_ROTATE_Z, ctrl, targ, angle);
    }
    void controlPhase(unsigned ctrl, unsigned targ, Fp angle)
    {
        gate2(QSLC_CONTROL_PHASE, ctrl, targ, angle);
    }
    void swap(unsigned q1, unsigned q2) { gate2(QSLC_SWAP, q1, q2); }
    void fswap(unsigned q1, unsigned q2) { gate2(QSLC_FSWAP, q1, q2); }
    void npRotateX(unsigned q1, unsigned q2, Fp angle) { gate2(QSLC_NP_ROTATE_X, q1, q2, angle); }
    void npRotateY(unsigned q1, unsigned q2, Fp angle) { gate2(QSLC_NP_ROTATE_Y, q1, q2, angle); }
    void npHadamard(unsigned q1, unsigned q2) { gate2(QSLC_NP_HADAMARD, q1, q2); }
};

/* Base plus the gates outside the number-preserving set
 * (HasNonNPGates, concepts.hpp:84-102). */
template <std::floating_point Fp>
class Full : public Base<Fp> {
public:
    // One-qubit gates (gates.cpp:32-209)
    void pauliX(unsigned targ) { this->gate1(QSLC_PAULI_X, targ); }
    void pauliY(unsigned targ) { this->gate1(QSLC_PAULI_Y, targ); }
    void hadamard(unsigned targ) { this->gate1(QSLC_HADAMARD, targ); }
    void rotateX(unsigned targ, Fp angle) { this->gate1(QSLC_ROTATE_X, targ, angle); }
    void rotateY(unsigned targ, Fp angle) { this->gate1(QSLC_ROTATE_Y, targ, angle); }
    // Controlled gates (gates.cpp:215-500)
    void controlNot(unsigned ctrl, unsigned targ) { this->gate2(QSLC_CONTROL_NOT, ctrl, targ); }
    void controlY(unsigned ctrl, unsigned targ) { this->gate2(QSLC_CONTROL_Y, ctrl, targ); }
    void controlRotateX(unsigned ctrl, unsigned targ, Fp angle)
    {
        this->gate2(QSLC_CONTROL_ROTATE_X, ctrl, targ, angle);
    }
    void controlRotateY(unsigned ctrl, unsigned targ, Fp angle)
    {
        this->gate2(QSLC_CONTROL_ROTATE_Y, ctrl, targ, angle);
    }
    void controlHadamard(unsigned ctrl, unsigned targ) { this->gate2(QSLC_CONTROL_HADAMARD, ctrl, targ); }
};

}  // namespace cuda_detail

/* Drop-in for Qubits<Type::Default, Fp> (default.hpp:65-713). */
template <std::floating_point Fp>
class Qubits<cuda_type, Fp> : public cuda_detail::Full<Fp> {
public:
    inline static const std::string name =
        std::is_same_v<Fp, double> ? "Qub<cuda,double>" : "Qub<cuda,float>";
    using Fp_type = Fp;

    /// The all-zero state (default.cpp:39-46).
    explicit Qubits(unsigned nqubits)
    {
        cuda_detail::check(qslc_create(nqubits, cuda_detail::dtype_of<Fp>, &this->h));
    }
    /// From a state vector (default.cpp:48-55).
    explicit Qubits(const std::vector<complex<Fp>> &state)
    {
        unsigned n = cuda_detail::log2_size(state.size());
        cuda_detail::check(qslc_create(n, cuda_detail::dtype_of<Fp>, &this->h));
        this->setState(state);
    }
    Qubits(const Qubits &) = default;
    Qubits(Qubits &&) noexcept = default;
    /// Copies the amplitudes; throws on a qubit-count mismatch (default.cpp:94-105).
    void operator=(const Qubits &old) { this->assign(old); }
};

/* Drop-in for Qubits<Type::Resize, Fp> (resize.hpp:46-370): the Default
 * gates and measurement on a state whose qubit count changes. */
template <std::floating_point Fp>
class Qubits<cuda_resize_type, Fp> : public cuda_detail::Full<Fp> {
public:
    inline static const std::string name =
        std::is_same_v<Fp, double> ? "Qub<cuda_resize,double>" : "Qub<cuda_resize,float>";
    using Fp_type = Fp;

    /// The all-zero state (resize.cpp:39-46).
    explicit Qubits(unsigned nqubits)
    {
        this->shared_rng = true;
        cuda_detail::check(qslc_create_resizable(nqubits, cuda_detail::dtype_of<Fp>, &this->h));
    }
    /// From a state vector of any power-of-two size (resize.cpp:48-55).
    explicit Qubits(const std::vector<complex<Fp>> &state)
    {
        this->shared_rng = true;
        unsigned n = cuda_detail::log2_size(state.size());
        cuda_detail::check(qslc_create_resizable(n, cuda_detail::dtype_of<Fp>, &this->h));
        this->setState(state);
    }
    Qubits(const Qubits &) = default;
    Qubits(Qubits &&) noexcept = default;
    /// Takes the other object's qubit count and amplitudes (the implicit
    /// assignment of resize.hpp; resize.cpp:150-165 is commented out).
    void operator=(const Qubits &old) { this->assign(old); }

    /// A qubit in |0> at position targ; the qubits at and above it move up
    /// by one (resize.cpp:106-147).
    void addQubit(unsigned targ) { cuda_detail::check(qslc_add_qubit(this->h, targ)); }
    /// addQubit(getNumQubits()) (resize.cpp:100-104).
    void appendQubit() { addQubit(this->getNumQubits()); }
    /// Trim the allocation to the live amplitudes (resize.cpp:92-98).
    void reallocateState() { cuda_detail::check(qslc_reallocate(this->h)); }

    /// measure and remove qubit targ (resize/measure.cpp:156-182)
    int measureOut(unsigned targ)
    {
        const Fp u = this->draw();
        int out = 0;
        cuda_detail::check(qslc_measure_out(this->h, targ, double(u), &out));
        return out;
    }
    /// postselect and remove qubit targ (resize/measure.cpp:238-251)
    Fp postselectOut(unsigned targ, unsigned outcome)
    {
        double p = 0;
        cuda_detail::check(qslc_postselect_out(this->h, targ, outcome, &p));
        return Fp(p);
    }
};

/* Drop-in for Qubits<Type::NP, Fp> (np.hpp:55-253): only the C(n, nones)
 * amplitudes of the preserved Hamming weight are stored on the device. */
template <std::floating_point Fp>
class Qubits<cuda_np_type, Fp> : public cuda_detail::Base<Fp> {
public:
    inline static const std::string name =
        std::is_same_v<Fp, double> ? "Qub<cuda_np,double>" : "Qub<cuda_np,float>";
    using Fp_type = Fp;

    /// The basis state with the nones lowest bits set; throws unless
    /// 1 <= nones < nqubits (np.cpp:42-55).
    explicit Qubits(unsigned nqubits, unsigned nones = 1)
    {
        cuda_detail::check(qslc_create_np(nqubits, nones, cuda_detail::dtype_of<Fp>, &this->h));
    }
    /// From a state vector; the weight comes from the state, which must
    /// have a single Hamming weight (np.cpp:57-65, quantum.cpp:133-156).
    explicit Qubits(const std::vector<complex<Fp>> &state)
    {
        unsigned n = cuda_detail::log2_size(state.size());
        cuda_detail::check(qslc_create_np(n, 1, cuda_detail::dtype_of<Fp>, &this->h));
        this->setState(state);
    }
    Qubits(const Qubits &) = default;
    Qubits(Qubits &&) noexcept = default;
    void operator=(const Qubits &old) { this->assign(old); }

    unsigned getNumOnes() const
    {
        unsigned w = 0;
        cuda_detail::check(qslc_num_ones(this->h, &w));
        return w;
    }
    void setNumOnes(unsigned nones) { cuda_detail::check(qslc_set_num_ones(this->h, nones)); }
};

}  // namespace qsl

#endif
