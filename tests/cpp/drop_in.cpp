// Runs a circuit through qsl::Qubits<qsl::cuda_type, Fp> -- the C++ drop-in,
// exactly as a qsl user would call it -- and writes what it observed so the
// Python test can compare it with the oracle.
//
// usage: drop_in <circuit.txt> <out.bin> <nqubits> <seed> <nshots> [f32]
// circuit.txt: one gate per line, "name q1 q2 angle" (q2 = -1 for one-qubit)
// out.bin: state (2^n complex), probs (n x 2 Fp), uniforms (nshots Fp),
//          sampleAll counts as (index, count) uint64 pairs, terminated by
//          the pair (2^64-1, 0).
#include <qsl/qubits/cuda.hpp>

#include <cstdio>
#include <fstream>
#include <functional>
#include <random>
#include <sstream>
#include <string>
#include <unordered_map>

template <class Fp>
int run(const char *circ, const char *out, unsigned n, unsigned seed, std::size_t nshots)
{
    using Q = qsl::Qubits<qsl::cuda_type, Fp>;
    Q q(n);
    std::unordered_map<std::string, std::function<void(unsigned, unsigned, Fp)>> g = {
        {"pauliX", [&](unsigned a, unsigned, Fp) { q.pauliX(a); }},
        {"pauliY", [&](unsigned a, unsigned, Fp) { q.pauliY(a); }},
        {"pauliZ", [&](unsigned a, unsigned, Fp) { q.pauliZ(a); }},
        {"hadamard", [&](unsigned a, unsigned, Fp) { q.hadamard(a); }},
        {"phase", [&](unsigned a, unsigned, Fp t) { q.phase(a, t); }},
        {"rotateX", [&](unsigned a, unsigned, Fp t) { q.rotateX(a, t); }},
        {"rotateY", [&](unsigned a, unsigned, Fp t) { q.rotateY(a, t); }},
        {"rotateZ", [&](unsigned a, unsigned, Fp t) { q.rotateZ(a, t); }},
        {"controlNot", [&](unsigned a, unsigned b, Fp) { q.controlNot(a, b); }},
        {"controlY", [&](unsigned a, unsigned b, Fp) { q.controlY(a, b); }},
        {"controlZ", [&](unsigned a, unsigned b, Fp) { q.controlZ(a, b); }},
        {"controlRotateX", [&](unsigned a, unsigned b, Fp t) { q.controlRotateX(a, b, t); }},
        {"controlRotateY", [&](unsigned a, unsigned b, Fp t) { q.controlRotateY(a, b, t); }},
        {"controlRotateZ", [&](unsigned a, unsigned b, Fp t) { q.controlRotateZ(a, b, t); }},
        {"controlPhase", [&](unsigned a, unsigned b, Fp t) { q.controlPhase(a, b, t); }},
        {"controlHadamard", [&](unsigned a, unsigned b, Fp) { q.controlHadamard(a, b); }},
        {"swap", [&](unsigned a, unsigned b, Fp) { q.swap(a, b); }},
        {"fswap", [&](unsigned a, unsigned b, Fp) { q.fswap(a, b); }},
        {"npRotateX", [&](unsigned a, unsigned b, Fp t) { q.npRotateX(a, b, t); }},
        {"npRotateY", [&](unsigned a, unsigned b, Fp t) { q.npRotateY(a, b, t); }},
        {"npHadamard", [&](unsigned a, unsigned b, Fp) { q.npHadamard(a, b); }},
    };
    std::ifstream in(circ);
    std::string line;
    while (std::getline(in, line)) {
        std::istringstream ss(line);
        std::string name;
        long a, b;
        double t;
        if (!(ss >> name >> a >> b >> t)) continue;
        g.at(name)(unsigned(a), unsigned(b < 0 ? 0 : b), Fp(t));
    }
    Q copy(q);                       // copy constructor: device-to-device
    auto st = copy.getState();
    std::ofstream o(out, std::ios::binary);
    o.write(reinterpret_cast<const char *>(st.data()), st.size() * sizeof(st[0]));
    for (unsigned t = 0; t < n; t++)
        for (unsigned v = 0; v < 2; v++) {
            Fp p = q.prob(t, v);
            o.write(reinterpret_cast<const char *>(&p), sizeof(p));
        }
    // the uniforms the object will draw: same engine and distribution
    std::mt19937 mirror(seed);
    std::uniform_real_distribution<Fp> dist(0, 1);
    for (std::size_t i = 0; i < nshots; i++) {
        Fp u = dist(mirror);
        o.write(reinterpret_cast<const char *>(&u), sizeof(u));
    }
    q.seed(seed);
    auto m = q.sampleAll(nshots);
    for (auto [k, c] : m) {
        std::uint64_t kk = k, cc = c;
        o.write(reinterpret_cast<const char *>(&kk), 8);
        o.write(reinterpret_cast<const char *>(&cc), 8);
    }
    std::uint64_t end = ~0ull, zero = 0;
    o.write(reinterpret_cast<const char *>(&end), 8);
    o.write(reinterpret_cast<const char *>(&zero), 8);
    // operator= across sizes throws std::logic_error, as in qsl
    Q other(n + 1);
    try {
        other = q;
        std::fprintf(stderr, "operator= did not throw\n");
        return 2;
    } catch (const std::logic_error &) {
    }
    return 0;
}

int main(int argc, char **argv)
{
    if (argc < 6) {
        std::fprintf(stderr, "usage: drop_in circuit out n seed nshots [f32]\n");
        return 1;
    }
    unsigned n = unsigned(std::stoul(argv[3])), seed = unsigned(std::stoul(argv[4]));
    std::size_t shots = std::stoull(argv[5]);
    try {
        if (argc > 6 && std::string(argv[6]) == "f32") return run<float>(argv[1], argv[2], n, seed, shots);
        return run<double>(argv[1], argv[2], n, seed, shots);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 3;
    }
}
