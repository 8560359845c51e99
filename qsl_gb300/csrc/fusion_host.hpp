// fusion_host.hpp -- gate fusion for the precision form (plain C++, host only).
//
// A run of gates whose qubits together number at most k is one unitary on
// a 2^k-dimensional subspace; applying that dense block once replaces one
// sweep over the state per gate.  The planner walks the circuit's
// dependency order (two gates depend on each other only through a shared
// qubit; gates on disjoint qubits commute) and greedily grows each block
// from the first gate not yet placed, adding ready gates while the block's
// qubit set stays within k, preferring gates that add no new qubit.
//
// Gate matrices follow qsl's definitions operation by operation
// (src/qubits/default/gates.cpp): e.g. rotateX maps (a0, a1) to
// (c a0 - i s a1, c a1 - i s a0) with c = cos(angle/2), s = sin(angle/2)
// (:139-144), pauliY maps (a0, a1) to (-i a1, i a0) (:59-62).
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <vector>

#include "qslc.h"

namespace qslc {

using cd = std::complex<double>;

struct GateOp {
    int code;
    unsigned q1, q2;   // q2 unused (== q1) for one-qubit gates
    double angle;
};

inline bool is_two_qubit(int code) { return code >= QSLC_CONTROL_NOT; }

// 2x2 matrix of a one-qubit gate, m[out][in], on (|0>, |1>) of the target.
inline void gate1_matrix(int code, double angle, cd m[2][2])
{
    const cd I(0, 1);
    const double c = std::cos(angle / 2), s = std::sin(angle / 2);
    m[0][0] = m[0][1] = m[1][0] = m[1][1] = 0;
    switch (code) {
    case QSLC_PAULI_X: m[0][1] = m[1][0] = 1; break;
    case QSLC_PAULI_Y: m[0][1] = -I; m[1][0] = I; break;
    case QSLC_PAULI_Z: m[0][0] = 1; m[1][1] = -1; break;
    case QSLC_HADAMARD: {
        const double r = 1 / std::sqrt(2.0);
        m[0][0] = m[0][1] = m[1][0] = r;
        m[1][1] = -r;
        break;
    }
    case QSLC_PHASE: m[0][0] = 1; m[1][1] = std::polar(1.0, angle); break;
    case QSLC_ROTATE_X: m[0][0] = m[1][1] = c; m[0][1] = m[1][0] = -I * s; break;
    case QSLC_ROTATE_Y: m[0][0] = m[1][1] = c; m[0][1] = -s; m[1][0] = s; break;
    case QSLC_ROTATE_Z: m[0][0] = cd(c, -s); m[1][1] = cd(c, s); break;
    default: break;
    }
}

// 4x4 matrix of a two-qubit gate on local index b1 + 2*b2 (b1: bit of q1,
// b2: bit of q2).  For the control* gates q1 is the control.
inline void gate2_matrix(int code, double angle, cd m[4][4])
{
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) m[i][j] = (i == j) ? 1 : 0;
    auto put2 = [&](int a, int b, const cd u[2][2]) {   // act on basis pair (a, b)
        m[a][a] = u[0][0]; m[a][b] = u[0][1];
        m[b][a] = u[1][0]; m[b][b] = u[1][1];
    };
    cd u[2][2];
    switch (code) {
    case QSLC_CONTROL_NOT: gate1_matrix(QSLC_PAULI_X, 0, u); put2(1, 3, u); break;
    case QSLC_CONTROL_Y: gate1_matrix(QSLC_PAULI_Y, 0, u); put2(1, 3, u); break;
    case QSLC_CONTROL_Z: m[3][3] = -1; break;
    case QSLC_CONTROL_ROTATE_X: gate1_matrix(QSLC_ROTATE_X, angle, u); put2(1, 3, u); break;
    case QSLC_CONTROL_ROTATE_Y: gate1_matrix(QSLC_ROTATE_Y, angle, u); put2(1, 3, u); break;
    case QSLC_CONTROL_ROTATE_Z: gate1_matrix(QSLC_ROTATE_Z, angle, u); put2(1, 3, u); break;
    case QSLC_CONTROL_PHASE: m[3][3] = std::polar(1.0, angle); break;
    case QSLC_CONTROL_HADAMARD: gate1_matrix(QSLC_HADAMARD, 0, u); put2(1, 3, u); break;
    case QSLC_SWAP: gate1_matrix(QSLC_PAULI_X, 0, u); put2(1, 2, u); break;
    case QSLC_FSWAP: gate1_matrix(QSLC_PAULI_X, 0, u); put2(1, 2, u); m[3][3] = -1; break;
    case QSLC_NP_ROTATE_X: gate1_matrix(QSLC_ROTATE_X, angle, u); put2(1, 2, u); break;
    case QSLC_NP_ROTATE_Y: gate1_matrix(QSLC_ROTATE_Y, angle, u); put2(1, 2, u); break;
    case QSLC_NP_HADAMARD: gate1_matrix(QSLC_HADAMARD, 0, u); put2(1, 2, u); break;
    default: break;
    }
}

// A fused block: `k` qubits (ascending), U[out * 2^k + in], local index bit
// j standing for qubit qubits[j].
struct Block {
    int k = 0;
    unsigned qubits[8] = {};
    std::vector<cd> U;
    int ngates = 0;
};

// Multiply a gate into a block: U <- G U (G acting on the local bits of its
// qubits), column by column.
inline void block_apply_gate(Block &b, const GateOp &g)
{
    const int dim = 1 << b.k;
    auto local = [&](unsigned q) {
        for (int j = 0; j < b.k; j++)
            if (b.qubits[j] == q) return j;
        return -1;
    };
    if (!is_two_qubit(g.code)) {
        cd m[2][2];
        gate1_matrix(g.code, g.angle, m);
        const int t = local(g.q1);
        for (int col = 0; col < dim; col++)
            for (int r = 0; r < dim; r++) {
                if (r & (1 << t)) continue;
                cd &a0 = b.U[size_t(r) * dim + col];
                cd &a1 = b.U[size_t(r | (1 << t)) * dim + col];
                const cd x0 = a0, x1 = a1;
                a0 = m[0][0] * x0 + m[0][1] * x1;
                a1 = m[1][0] * x0 + m[1][1] * x1;
            }
    } else {
        cd m[4][4];
        gate2_matrix(g.code, g.angle, m);
        const int t1 = local(g.q1), t2 = local(g.q2);
        for (int col = 0; col < dim; col++)
            for (int r = 0; r < dim; r++) {
                if (r & ((1 << t1) | (1 << t2))) continue;
                cd *p[4];
                cd x[4];
                for (int v = 0; v < 4; v++) {
                    int row = r | ((v & 1) << t1) | (((v >> 1) & 1) << t2);
                    p[v] = &b.U[size_t(row) * dim + col];
                    x[v] = *p[v];
                }
                for (int o = 0; o < 4; o++) {
                    cd acc = 0;
                    for (int v = 0; v < 4; v++) acc += m[o][v] * x[v];
                    *p[o] = acc;
                }
            }
    }
    b.ngates++;
}

// Plan blocks of at most `kmax` qubits for `gates` (in circuit order).
inline std::vector<Block> plan_blocks(const std::vector<GateOp> &gates, int kmax, unsigned nqubits)
{
    const size_t n = gates.size();
    // per qubit, the gates that touch it, in order; frontier = next unplaced
    std::vector<std::vector<uint32_t>> on(nqubits);
    for (size_t i = 0; i < n; i++) {
        on[gates[i].q1].push_back(uint32_t(i));
        if (is_two_qubit(gates[i].code)) on[gates[i].q2].push_back(uint32_t(i));
    }
    std::vector<size_t> front(nqubits, 0);
    std::vector<char> placed(n, 0);
    auto ready = [&](size_t i) {
        const GateOp &g = gates[i];
        if (on[g.q1][front[g.q1]] != i) return false;
        if (is_two_qubit(g.code) && on[g.q2][front[g.q2]] != i) return false;
        return true;
    };
    auto place = [&](size_t i) {
        placed[i] = 1;
        front[gates[i].q1]++;
        if (is_two_qubit(gates[i].code)) front[gates[i].q2]++;
    };
    std::vector<Block> out;
    size_t first = 0;
    std::vector<unsigned> S;
    std::vector<size_t> members;
    while (true) {
        while (first < n && placed[first]) first++;
        if (first >= n) break;
        S.clear();
        members.clear();
        auto add = [&](size_t i) {
            const GateOp &g = gates[i];
            if (std::find(S.begin(), S.end(), g.q1) == S.end()) S.push_back(g.q1);
            if (is_two_qubit(g.code) && std::find(S.begin(), S.end(), g.q2) == S.end()) S.push_back(g.q2);
            members.push_back(i);
            place(i);
        };
        add(first);
        // grow: gates ready at the frontier of qubits in S first, then any
        // ready gate whose qubits fit
        bool grew = true;
        while (grew) {
            grew = false;
            for (size_t si = 0; si < S.size(); si++) {
                const unsigned q = S[si];
                while (front[q] < on[q].size()) {
                    const size_t i = on[q][front[q]];
                    if (!ready(i)) break;
                    const GateOp &g = gates[i];
                    const unsigned other = is_two_qubit(g.code) ? (g.q1 == q ? g.q2 : g.q1) : q;
                    const bool has = std::find(S.begin(), S.end(), other) != S.end();
                    if (!has && int(S.size()) + 1 > kmax) break;
                    add(i);
                    grew = true;
                }
            }
            if (grew) continue;
            // bring in one new qubit: the earliest ready gate that fits
            for (size_t i = first; i < n && int(S.size()) < kmax; i++) {
                if (placed[i] || !ready(i)) continue;
                const GateOp &g = gates[i];
                int extra = 0;
                if (std::find(S.begin(), S.end(), g.q1) == S.end()) extra++;
                if (is_two_qubit(g.code) && std::find(S.begin(), S.end(), g.q2) == S.end()) extra++;
                if (int(S.size()) + extra > kmax) continue;
                add(i);
                grew = true;
                break;
            }
        }
        Block b;
        std::sort(S.begin(), S.end());
        b.k = int(S.size());
        for (int j = 0; j < b.k; j++) b.qubits[j] = S[j];
        const int dim = 1 << b.k;
        b.U.assign(size_t(dim) * dim, cd(0));
        for (int j = 0; j < dim; j++) b.U[size_t(j) * dim + j] = 1;
        for (size_t i : members) block_apply_gate(b, gates[i]);
        out.push_back(std::move(b));
    }
    return out;
}

}  // namespace qslc
