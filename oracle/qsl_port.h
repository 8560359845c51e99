/*
 * qsl_port.h -- declarations of the oracle (CPU restatement of qsl's
 * Default / OpenMP / NP amplitude loops).  Test infrastructure only.
 *
 * Suffix _d works on interleaved double {re, im} arrays, _f on float.
 * `nth` is the OpenMP thread count (1 = the serial Default backend).
 */
#ifndef QSL_PORT_H
#define QSL_PORT_H
#include <stddef.h>
#include <stdint.h>

/* op codes of port_*_gate2 (Default two-qubit gates, gates.cpp:215-682);
 * for the controlled ops q1 is the control and q2 the target */
enum {
    OP2_CNOT, OP2_CY, OP2_CZ, OP2_CRX, OP2_CRY, OP2_CRZ, OP2_CPHASE, OP2_CH,
    OP2_SWAP, OP2_FSWAP, OP2_NPRX, OP2_NPRY, OP2_NPH
};

/* op codes of port_*_np_gate2 (np/gates.cpp:118-415) */
enum {
    NP2_CZ, NP2_CPHASE, NP2_CRZ01, NP2_SWAP, NP2_NPRX, NP2_NPRY, NP2_NPH
};

#define PORT_DECL(FP, SFX)                                                    \
    void port_##SFX##_pauliX(FP *s, unsigned n, unsigned targ, int nth);      \
    void port_##SFX##_pauliY(FP *s, unsigned n, unsigned targ, int nth);      \
    void port_##SFX##_pauliZ(FP *s, unsigned n, unsigned targ, int nth);      \
    void port_##SFX##_hadamard(FP *s, unsigned n, unsigned targ, int nth);    \
    void port_##SFX##_phase(FP *s, unsigned n, unsigned targ, FP a, int nth); \
    void port_##SFX##_rotateX(FP *s, unsigned n, unsigned targ, FP a, int nth); \
    void port_##SFX##_rotateY(FP *s, unsigned n, unsigned targ, FP a, int nth); \
    void port_##SFX##_rotateZ(FP *s, unsigned n, unsigned targ, FP a, int nth); \
    void port_##SFX##_gate2(FP *s, unsigned n, int op, unsigned q1,           \
                            unsigned q2, FP a, int nth);                      \
    FP port_##SFX##_prob(const FP *s, unsigned n, unsigned targ, unsigned o); \
    FP port_##SFX##_prob_omp(const FP *s, unsigned n, unsigned targ,          \
                             unsigned o, int nth);                            \
    void port_##SFX##_collapse(FP *s, unsigned n, unsigned targ, unsigned o,  \
                               FP factor, int nth);                           \
    int port_##SFX##_measure(FP *s, unsigned n, unsigned targ, FP u);         \
    FP port_##SFX##_postselect(FP *s, unsigned n, unsigned targ, unsigned o); \
    size_t port_##SFX##_generate_dist(const FP *s, unsigned n, uint64_t *idx, \
                                      double *cdf);                           \
    uint64_t port_##SFX##_draw_sample(const uint64_t *idx, const double *cdf, \
                                      size_t m, FP u);                        \
    uint64_t port_##SFX##_measure_all(FP *s, unsigned n, FP u,                \
                                      uint64_t *idx, double *cdf);            \
    void port_##SFX##_sample_all(const FP *s, unsigned n, const FP *u,        \
                                 size_t nshots, uint64_t *out, uint64_t *idx, \
                                 double *cdf);                                \
    void port_##SFX##_sample(const FP *s, unsigned n, unsigned targ,          \
                             const FP *u, size_t nshots, uint64_t counts[2]); \
    void port_##SFX##_sample_all2(const FP *s, unsigned n, const FP *u_sorted,\
                                  size_t nshots, uint64_t *counts);           \
    void port_##SFX##_add_qubit(FP *s, unsigned n, unsigned targ);            \
    void port_##SFX##_collapse_out(FP *s, unsigned n, unsigned targ,          \
                                   unsigned o, FP factor);                    \
    void port_##SFX##_np_phase1(FP *s, const uint64_t *tab, size_t len,       \
                                unsigned targ, int mode, FP a, int nth);      \
    void port_##SFX##_np_rz0(FP *s, const uint64_t *tab, size_t len,          \
                             unsigned targ, FP a, int nth);                   \
    void port_##SFX##_np_gate2(FP *s, const uint64_t *tab, size_t len, int op,\
                               unsigned q1, unsigned q2, FP a, int nth);      \
    FP port_##SFX##_np_prob(const FP *s, const uint64_t *tab, size_t len,     \
                            unsigned targ, unsigned o);                       \
    void port_##SFX##_np_collapse(FP *s, const uint64_t *tk, size_t lk,       \
                                  const uint64_t *tz, size_t lz,              \
                                  unsigned targ, unsigned o, FP factor);      \
    size_t port_##SFX##_np_generate_dist(const FP *s, const uint64_t *tab,    \
                                         size_t len, uint64_t *idx,           \
                                         double *cdf);                        \
    void port_##SFX##_np_sample_all2(const FP *s, const uint64_t *tab,        \
                                     size_t len, const FP *u_sorted,          \
                                     size_t nshots, uint64_t *counts);

PORT_DECL(double, d)
PORT_DECL(float, f)

uint64_t port_next(uint64_t x);
unsigned port_hamming_weight(uint64_t n);
unsigned port_choose(unsigned n, unsigned k);
size_t port_generate_lookup(unsigned len, unsigned ones, uint64_t *out,
                            size_t cap);
int port_check_state_np_d(const double *s, unsigned n);
int port_num_threads(void);

#endif
