// Checks the fusion planner (qsl_gb300/csrc/fusion_host.hpp):
//  1. every gate matrix acts on a state as the oracle's restatement of the
//     reference's loop does (to 1e-13: the loop rounds differently);
//  2. applying the planned blocks equals applying the gates one by one, for
//     random circuits of every gate, block sizes 1..5;
//  3. every block respects its size limit and the blocks hold every gate.
#include "fusion_host.hpp"

extern "C" {
#include "qsl_port.h"
}

#include <cstdio>
#include <random>

using namespace qslc;

static std::mt19937_64 rng(7);

static void apply_block(std::vector<cd> &st, unsigned n, const Block &b)
{
    const size_t dim = size_t(1) << n;
    const int kd = 1 << b.k;
    std::vector<cd> in(kd), out(kd);
    for (size_t base = 0; base < dim; base++) {
        bool zero = true;
        for (int j = 0; j < b.k; j++)
            if (base & (size_t(1) << b.qubits[j])) zero = false;
        if (!zero) continue;
        for (int v = 0; v < kd; v++) {
            size_t idx = base;
            for (int j = 0; j < b.k; j++)
                if (v & (1 << j)) idx |= size_t(1) << b.qubits[j];
            in[v] = st[idx];
        }
        for (int o = 0; o < kd; o++) {
            cd acc = 0;
            for (int v = 0; v < kd; v++) acc += b.U[size_t(o) * kd + v] * in[v];
            out[o] = acc;
        }
        for (int v = 0; v < kd; v++) {
            size_t idx = base;
            for (int j = 0; j < b.k; j++)
                if (v & (1 << j)) idx |= size_t(1) << b.qubits[j];
            st[idx] = out[v];
        }
    }
}

static void port_gate(std::vector<cd> &st, unsigned n, const GateOp &g)
{
    double *s = reinterpret_cast<double *>(st.data());
    switch (g.code) {
    case QSLC_PAULI_X: port_d_pauliX(s, n, g.q1, 1); return;
    case QSLC_PAULI_Y: port_d_pauliY(s, n, g.q1, 1); return;
    case QSLC_PAULI_Z: port_d_pauliZ(s, n, g.q1, 1); return;
    case QSLC_HADAMARD: port_d_hadamard(s, n, g.q1, 1); return;
    case QSLC_PHASE: port_d_phase(s, n, g.q1, g.angle, 1); return;
    case QSLC_ROTATE_X: port_d_rotateX(s, n, g.q1, g.angle, 1); return;
    case QSLC_ROTATE_Y: port_d_rotateY(s, n, g.q1, g.angle, 1); return;
    case QSLC_ROTATE_Z: port_d_rotateZ(s, n, g.q1, g.angle, 1); return;
    default: break;
    }
    static const int op2[] = {OP2_CNOT, OP2_CY, OP2_CZ, OP2_CRX, OP2_CRY, OP2_CRZ, OP2_CPHASE,
                              OP2_CH, OP2_SWAP, OP2_FSWAP, OP2_NPRX, OP2_NPRY, OP2_NPH};
    port_d_gate2(s, n, op2[g.code - QSLC_CONTROL_NOT], g.q1, g.q2, g.angle, 1);
}

static GateOp random_gate(unsigned n)
{
    static const int codes[] = {0, 1, 2, 3, 4, 5, 6, 7, 16, 17, 18, 19, 20, 21, 22, 23, 24, 25, 26, 27, 28};
    GateOp g{};
    g.code = codes[rng() % 21];
    g.q1 = unsigned(rng() % n);
    g.q2 = g.q1;
    if (is_two_qubit(g.code))
        while (g.q2 == g.q1) g.q2 = unsigned(rng() % n);
    g.angle = std::uniform_real_distribution<double>(0, 6.283185307179586)(rng);
    return g;
}

static std::vector<cd> random_state(unsigned n)
{
    std::normal_distribution<double> d;
    std::vector<cd> v(size_t(1) << n);
    double nrm = 0;
    for (auto &x : v) {
        x = cd(d(rng), d(rng));
        nrm += std::norm(x);
    }
    for (auto &x : v) x /= std::sqrt(nrm);
    return v;
}

static double maxdiff(const std::vector<cd> &a, const std::vector<cd> &b)
{
    double m = 0;
    for (size_t i = 0; i < a.size(); i++) m = std::max(m, std::abs(a[i] - b[i]));
    return m;
}

int main()
{
    int fails = 0;
    // 1. single-gate matrices against the oracle
    for (int t = 0; t < 2000; t++) {
        unsigned n = 2 + unsigned(rng() % 5);
        GateOp g = random_gate(n);
        auto a = random_state(n), b = a;
        port_gate(a, n, g);
        std::vector<GateOp> one{g};
        for (const Block &bl : plan_blocks(one, 5, n)) apply_block(b, n, bl);
        if (maxdiff(a, b) > 1e-13) {
            if (fails++ < 10) std::printf("gate %d on (%u,%u): diff %g\n", g.code, g.q1, g.q2, maxdiff(a, b));
        }
    }
    // 2./3. circuits
    for (int t = 0; t < 300; t++) {
        unsigned n = 3 + unsigned(rng() % 7);
        int kmax = 1 + int(rng() % 5);
        std::vector<GateOp> circ;
        size_t len = 20 + rng() % 120;
        for (size_t i = 0; i < len; i++) {
            GateOp g = random_gate(n);
            if (kmax == 1 && is_two_qubit(g.code)) g.code = QSLC_ROTATE_X;
            circ.push_back(g);
        }
        auto a = random_state(n), b = a;
        for (const GateOp &g : circ) port_gate(a, n, g);
        auto blocks = plan_blocks(circ, std::max(kmax, 2), n);
        size_t total = 0;
        for (const Block &bl : blocks) {
            if (bl.k > std::max(kmax, 2)) fails++;
            total += size_t(bl.ngates);
            apply_block(b, n, bl);
        }
        if (total != circ.size()) {
            if (fails++ < 10) std::printf("blocks hold %zu of %zu gates\n", total, circ.size());
        }
        if (maxdiff(a, b) > 1e-11) {
            if (fails++ < 10) std::printf("circuit n=%u k=%d len=%zu diff %g\n", n, kmax, len, maxdiff(a, b));
        }
    }
    if (fails) return 1;
    std::puts("fusion ok");
    return 0;
}
