// ref_capi.cpp -- a C interface to the reference's own simulator classes.
//
// TEST INFRASTRUCTURE ONLY.  Built (by oracle/Makefile, target `ref`) into
// oracle/_ref/libqslref.so together with the reference's unmodified
// src/qubits/*/*.cpp and src/utils/*.cpp (minus random.cpp, replaced by
// ref_shim_random.cpp).  Python loads it through ctypes to pin the C
// restatement (qsl_port.c) and to write the golden fixtures in tests/golden.
//
// Every entry point forwards to one public member of
// qsl::Qubits<Type, Fp> (include/qsl/qubits/default.hpp:97-712,
// np.hpp:100-250); logic_error throws come back as negative return codes.
#include <cstdint>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include <cmath>   // results.tpp uses std::pow without including it
#include "qsl/benchmark/results.hpp"
#include "qsl/qubits.hpp"
#include "qsl/utils/misc.hpp"
#include "qsl/utils/quantum.hpp"

namespace {

enum Kind { K_DEFAULT = 0, K_OMP = 1, K_NP = 2, K_OMPNP = 3, K_RESIZE = 4 };

struct Base {
    virtual ~Base() = default;
    virtual Base *clone() const = 0;
    virtual int assign(const Base *other) = 0;
    virtual std::size_t dim() const = 0;
    virtual void get_state(void *out) const = 0;
    virtual int set_state(const void *in, std::size_t dim) = 0;
    virtual int gate(const std::string &name, unsigned q1, unsigned q2, double a) = 0;
    virtual double prob(unsigned t, unsigned o) const = 0;
    virtual int measure(unsigned t) = 0;
    virtual double postselect(unsigned t, unsigned o) = 0;
    virtual std::uint64_t measure_all() = 0;
    virtual std::map<std::size_t, std::size_t> sample_all(std::size_t n) = 0;
    virtual std::map<std::size_t, std::size_t> sample_all2(std::size_t n) = 0;
    virtual std::vector<std::size_t> sample(unsigned t, std::size_t n) = 0;
    virtual void reset() = 0;
    virtual int set_basis(std::uint64_t idx) = 0;
    virtual int num_ones() const = 0;
    virtual int set_num_ones(unsigned w) = 0;
    virtual unsigned num_qubits() const = 0;
    // Resize backend only (resize.hpp:160-180, :310, :350); -2 elsewhere
    virtual int add_qubit(unsigned t) = 0;
    virtual int append_qubit() = 0;
    virtual int measure_out(unsigned t) = 0;
    virtual double postselect_out(unsigned t, unsigned o) = 0;
    virtual int reallocate() = 0;
};

template <class S>
struct Impl final : Base {
    using Fp = typename S::Fp_type;
    S sim;
    template <class... A>
    explicit Impl(A &&...a) : sim(std::forward<A>(a)...) {}
    Impl(const Impl &o) : sim(o.sim) {}

    Base *clone() const override { return new Impl(*this); }
    int assign(const Base *other) override
    {
        auto *o = dynamic_cast<const Impl *>(other);
        if (!o) return -3;
        try { sim = o->sim; } catch (const std::logic_error &) { return -1; }
        return 0;
    }
    std::size_t dim() const override { return std::size_t(1) << sim.getNumQubits(); }
    void get_state(void *out) const override
    {
        auto st = sim.getState();
        std::memcpy(out, st.data(), st.size() * sizeof(qsl::complex<Fp>));
    }
    int set_state(const void *in, std::size_t d) override
    {
        std::vector<qsl::complex<Fp>> v(d);
        std::memcpy(v.data(), in, d * sizeof(qsl::complex<Fp>));
        try { sim.setState(v); } catch (const std::logic_error &) { return -1; }
        return 0;
    }
    int gate(const std::string &g, unsigned q1, unsigned q2, double a) override
    {
        Fp t = static_cast<Fp>(a);
        // Gates every backend has (HasNPGates, concepts.hpp:65-82)
        if (g == "pauliZ") { sim.pauliZ(q1); return 0; }
        if (g == "rotateZ") { sim.rotateZ(q1, t); return 0; }
        if (g == "phase") { sim.phase(q1, t); return 0; }
        if (g == "controlZ") { sim.controlZ(q1, q2); return 0; }
        if (g == "controlRotateZ") { sim.controlRotateZ(q1, q2, t); return 0; }
        if (g == "controlPhase") { sim.controlPhase(q1, q2, t); return 0; }
        if (g == "swap") { sim.swap(q1, q2); return 0; }
        if (g == "fswap") { sim.fswap(q1, q2); return 0; }
        if (g == "npRotateX") { sim.npRotateX(q1, q2, t); return 0; }
        if (g == "npRotateY") { sim.npRotateY(q1, q2, t); return 0; }
        if (g == "npHadamard") { sim.npHadamard(q1, q2); return 0; }
        // Gates outside the number-preserving set (HasNonNPGates, :84-102)
        if constexpr (qsl::HasNonNPGates<S>) {
            if (g == "pauliX") { sim.pauliX(q1); return 0; }
            if (g == "pauliY") { sim.pauliY(q1); return 0; }
            if (g == "rotateX") { sim.rotateX(q1, t); return 0; }
            if (g == "rotateY") { sim.rotateY(q1, t); return 0; }
            if (g == "hadamard") { sim.hadamard(q1); return 0; }
            if (g == "controlNot") { sim.controlNot(q1, q2); return 0; }
            if (g == "controlY") { sim.controlY(q1, q2); return 0; }
            if (g == "controlRotateX") { sim.controlRotateX(q1, q2, t); return 0; }
            if (g == "controlRotateY") { sim.controlRotateY(q1, q2, t); return 0; }
            if (g == "controlHadamard") { sim.controlHadamard(q1, q2); return 0; }
        }
        return -2;
    }
    double prob(unsigned t, unsigned o) const override { return sim.prob(t, o); }
    int measure(unsigned t) override { return sim.measure(t); }
    double postselect(unsigned t, unsigned o) override { return sim.postselect(t, o); }
    std::uint64_t measure_all() override { return sim.measureAll(); }
    std::map<std::size_t, std::size_t> sample_all(std::size_t n) override { return sim.sampleAll(n); }
    std::map<std::size_t, std::size_t> sample_all2(std::size_t n) override
    {
        if constexpr (requires(S &s) { s.sampleAll2(n); }) return sim.sampleAll2(n);
        return {};
    }
    std::vector<std::size_t> sample(unsigned t, std::size_t n) override { return sim.sample(t, n); }
    void reset() override { sim.reset(); }
    int set_basis(std::uint64_t idx) override
    {
        try { sim.setBasisState(idx); } catch (const std::logic_error &) { return -1; }
        return 0;
    }
    int num_ones() const override
    {
        if constexpr (requires(const S &s) { s.getNumOnes(); }) return (int)sim.getNumOnes();
        return -1;
    }
    int set_num_ones(unsigned w) override
    {
        if constexpr (requires(S &s) { s.setNumOnes(1u); }) {
            try { sim.setNumOnes(w); } catch (const std::logic_error &) { return -1; }
            return 0;
        }
        return -2;
    }
    unsigned num_qubits() const override { return sim.getNumQubits(); }
    int add_qubit(unsigned t) override
    {
        if constexpr (requires(S &s) { s.addQubit(0u); }) { sim.addQubit(t); return 0; }
        return -2;
    }
    int append_qubit() override
    {
        if constexpr (requires(S &s) { s.appendQubit(); }) { sim.appendQubit(); return 0; }
        return -2;
    }
    int measure_out(unsigned t) override
    {
        if constexpr (requires(S &s) { s.measureOut(0u); }) return sim.measureOut(t);
        return -2;
    }
    double postselect_out(unsigned t, unsigned o) override
    {
        if constexpr (requires(S &s) { s.postselectOut(0u, 0u); }) return sim.postselectOut(t, o);
        return -2;
    }
    int reallocate() override
    {
        if constexpr (requires(S &s) { s.reallocateState(); }) { sim.reallocateState(); return 0; }
        return -2;
    }
};

template <class Fp>
std::vector<qsl::complex<Fp>> to_vec(const void *in, std::size_t d)
{
    std::vector<qsl::complex<Fp>> v(d);
    std::memcpy(v.data(), in, d * sizeof(qsl::complex<Fp>));
    return v;
}

template <class Fp>
Base *make(int kind, unsigned n, unsigned nones, unsigned nth)
{
    switch (kind) {
    case K_DEFAULT: return new Impl<qsl::Qubits<qsl::Type::Default, Fp>>(n);
    case K_OMP: return new Impl<qsl::Qubits<qsl::Type::Omp, Fp>>(n, nth);
    case K_NP: return new Impl<qsl::Qubits<qsl::Type::NP, Fp>>(n, nones);
    case K_OMPNP: return new Impl<qsl::Qubits<qsl::Type::OmpNP, Fp>>(n, nones, nth);
    case K_RESIZE: return new Impl<qsl::Qubits<qsl::Type::Resize, Fp>>(n);
    }
    return nullptr;
}

template <class Fp>
Base *make_from(int kind, const void *in, std::size_t d, unsigned nth)
{
    auto v = to_vec<Fp>(in, d);
    switch (kind) {
    case K_DEFAULT: return new Impl<qsl::Qubits<qsl::Type::Default, Fp>>(v);
    case K_OMP: return new Impl<qsl::Qubits<qsl::Type::Omp, Fp>>(v, nth);
    case K_NP: return new Impl<qsl::Qubits<qsl::Type::NP, Fp>>(v);
    case K_OMPNP: return new Impl<qsl::Qubits<qsl::Type::OmpNP, Fp>>(v, nth);
    case K_RESIZE: return new Impl<qsl::Qubits<qsl::Type::Resize, Fp>>(v);
    }
    return nullptr;
}

std::size_t dump_map(const std::map<std::size_t, std::size_t> &m, std::uint64_t *keys,
                     std::uint64_t *counts, std::size_t cap)
{
    std::size_t i = 0;
    for (const auto &[k, c] : m) {
        if (i < cap) { keys[i] = k; counts[i] = c; }
        i++;
    }
    return i;
}

}  // namespace

extern "C" {

void *qslref_create(int kind, int fp32, unsigned n, unsigned nones, unsigned nth)
{
    try {
        return fp32 ? make<float>(kind, n, nones, nth) : make<double>(kind, n, nones, nth);
    } catch (const std::logic_error &) {
        return nullptr;
    }
}

void *qslref_create_from_state(int kind, int fp32, const void *state, std::size_t dim,
                               unsigned nth)
{
    try {
        return fp32 ? make_from<float>(kind, state, dim, nth)
                    : make_from<double>(kind, state, dim, nth);
    } catch (const std::logic_error &) {
        return nullptr;
    }
}

void qslref_destroy(void *h) { delete static_cast<Base *>(h); }
void *qslref_clone(void *h) { return static_cast<Base *>(h)->clone(); }
int qslref_assign(void *dst, void *src)
{
    return static_cast<Base *>(dst)->assign(static_cast<Base *>(src));
}
std::size_t qslref_dim(void *h) { return static_cast<Base *>(h)->dim(); }
unsigned qslref_num_qubits(void *h) { return static_cast<Base *>(h)->num_qubits(); }
void qslref_get_state(void *h, void *out) { static_cast<Base *>(h)->get_state(out); }
int qslref_set_state(void *h, const void *in, std::size_t dim)
{
    return static_cast<Base *>(h)->set_state(in, dim);
}
int qslref_gate(void *h, const char *name, unsigned q1, unsigned q2, double angle)
{
    return static_cast<Base *>(h)->gate(name, q1, q2, angle);
}
double qslref_prob(void *h, unsigned t, unsigned o) { return static_cast<Base *>(h)->prob(t, o); }
int qslref_measure(void *h, unsigned t) { return static_cast<Base *>(h)->measure(t); }
double qslref_postselect(void *h, unsigned t, unsigned o)
{
    return static_cast<Base *>(h)->postselect(t, o);
}
std::uint64_t qslref_measure_all(void *h) { return static_cast<Base *>(h)->measure_all(); }
std::size_t qslref_sample_all(void *h, std::size_t n, std::uint64_t *keys, std::uint64_t *counts,
                              std::size_t cap)
{
    return dump_map(static_cast<Base *>(h)->sample_all(n), keys, counts, cap);
}
std::size_t qslref_sample_all2(void *h, std::size_t n, std::uint64_t *keys,
                               std::uint64_t *counts, std::size_t cap)
{
    return dump_map(static_cast<Base *>(h)->sample_all2(n), keys, counts, cap);
}
void qslref_sample(void *h, unsigned t, std::size_t n, std::uint64_t *counts)
{
    auto v = static_cast<Base *>(h)->sample(t, n);
    counts[0] = v[0];
    counts[1] = v[1];
}
void qslref_reset(void *h) { static_cast<Base *>(h)->reset(); }
int qslref_set_basis(void *h, std::uint64_t idx) { return static_cast<Base *>(h)->set_basis(idx); }
int qslref_num_ones(void *h) { return static_cast<Base *>(h)->num_ones(); }
int qslref_set_num_ones(void *h, unsigned w) { return static_cast<Base *>(h)->set_num_ones(w); }
int qslref_add_qubit(void *h, unsigned t) { return static_cast<Base *>(h)->add_qubit(t); }
int qslref_append_qubit(void *h) { return static_cast<Base *>(h)->append_qubit(); }
int qslref_measure_out(void *h, unsigned t) { return static_cast<Base *>(h)->measure_out(t); }
double qslref_postselect_out(void *h, unsigned t, unsigned o)
{
    return static_cast<Base *>(h)->postselect_out(t, o);
}
int qslref_reallocate(void *h) { return static_cast<Base *>(h)->reallocate(); }

// src/utils/misc.cpp
std::uint64_t qslref_next(std::uint64_t x)
{
    std::size_t v = x;
    qsl::next(v);
    return v;
}
unsigned qslref_hamming_weight(std::uint64_t x) { return qsl::hammingWeight(x); }
unsigned qslref_choose(unsigned n, unsigned k) { return qsl::choose(n, k); }
std::size_t qslref_generate_lookup(unsigned len, unsigned ones, std::uint64_t *out,
                                   std::size_t cap)
{
    auto v = qsl::generateLookup(len, ones);
    for (std::size_t i = 0; i < v.size() && i < cap; i++) out[i] = v[i];
    return v.size();
}

// include/qsl/benchmark/results.tpp: a Results<unsigned, double> of nrows
// rows (nint integer then nfp floating-point columns, row-major), headings
// and metadata as '\n'-separated lists, written by writeToFile.
int qslref_results_write(const char *path, const char *headings, const char *meta,
                         std::size_t nrows, std::size_t nint, const unsigned *ints, std::size_t nfp,
                         const double *fps)
{
    auto split = [](const char *s) {
        std::vector<std::string> out;
        std::string cur;
        for (; *s; s++) {
            if (*s == '\n') { out.push_back(cur); cur.clear(); }
            else cur += *s;
        }
        if (!cur.empty()) out.push_back(cur);
        return out;
    };
    try {
        qsl::Results<unsigned, double> r{split(headings)};
        for (const auto &m : split(meta)) r.addMeta(m);
        for (std::size_t i = 0; i < nrows; i++)
            r.addRow(std::vector<unsigned>(ints + i * nint, ints + (i + 1) * nint),
                     std::vector<double>(fps + i * nfp, fps + (i + 1) * nfp));
        r.writeToFile(path);
    } catch (const std::logic_error &) {
        return -1;
    }
    return 0;
}

// src/utils/quantum.cpp
int qslref_check_state_np(const double *state, std::size_t dim)
{
    try {
        return (int)qsl::checkStateNP(to_vec<double>(state, dim));
    } catch (const std::logic_error &) {
        return -1;
    }
}
int qslref_check_state_size(std::size_t dim)
{
    try {
        return (int)qsl::checkStateSize(std::vector<qsl::complex<double>>(dim));
    } catch (const std::logic_error &) {
        return -1;
    }
}
double qslref_fubini_study(const double *a, const double *b, std::size_t dim)
{
    return qsl::fubiniStudy(to_vec<double>(a, dim), to_vec<double>(b, dim));
}

}  // extern "C"
