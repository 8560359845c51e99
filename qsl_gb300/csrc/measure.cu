// measure.cu -- prob and sampleAll of the plain 2^n layout.
//
// Both are the reference's sequential sums, reproduced bit for bit by the
// tile machinery of seqsum.cuh:
//   prob(targ, outcome): Fp running sum over the amplitudes whose bit targ
//     is `outcome`, ascending (src/qubits/default/measure.cpp:126-147);
//   sampleAll / measureAll: double running sum over all amplitudes
//     (Dist::prob is double, default.hpp:74-77; measure.cpp:60-78), searched
//     once per uniform (measure.cpp:164-188).
#include "seqsum.cuh"

namespace qslc {

// T: amplitude type; A: the running sum (Fp in the reference; double in
// the precision form, which keeps norms in FP64)
template <class T, class A>
static int prob_t(qslc_state *s, unsigned targ, unsigned outcome, double *out)
{
    ProdHalf<T> pr{static_cast<const cplx<T> *>(s->amps), targ, uint64_t(outcome) << targ};
    SeqOut<A> so;
    int rc = seq_run<ProdHalf<T>, T, A>(s, pr, uint64_t(1) << (s->n - 1), false, so);
    if (rc) return rc;
    *out = double(so.total);
    return QSLC_OK;
}

int seq_prob(qslc_state *s, unsigned targ, unsigned outcome, double *out)
{
    if (s->dtype == QSLC_C128) return prob_t<double, double>(s, targ, outcome, out);
    if (s->fuse_k) return prob_t<float, double>(s, targ, outcome, out);
    return prob_t<float, float>(s, targ, outcome, out);
}

template <class T>
static int sample_all_t(qslc_state *s, const double *u, uint64_t n, uint64_t *out)
{
    ProdAll<T> pr{static_cast<const cplx<T> *>(s->amps)};
    auto host_index = [](uint64_t j) { return j; };
    return seq_sample<ProdAll<T>, T, double>(s, pr, uint64_t(1) << s->n, u, n, out, host_index);
}

// sampleAll2 (measure.cpp:237-267): an Fp running sum, strict comparison
template <class T>
static int sample_all2_t(qslc_state *s, const double *u, uint64_t n, uint64_t *out)
{
    ProdAll<T> pr{static_cast<const cplx<T> *>(s->amps)};
    auto host_index = [](uint64_t j) { return j; };
    return seq_sample<ProdAll<T>, T, T>(s, pr, uint64_t(1) << s->n, u, n, out, host_index, true);
}

int seq_sample_all2(qslc_state *s, const double *u, uint64_t n, uint64_t *out)
{
    return s->dtype == QSLC_C128 ? sample_all2_t<double>(s, u, n, out)
                                 : sample_all2_t<float>(s, u, n, out);
}

int seq_sample_all(qslc_state *s, const double *u, uint64_t n, uint64_t *out)
{
    return s->dtype == QSLC_C128 ? sample_all_t<double>(s, u, n, out)
                                 : sample_all_t<float>(s, u, n, out);
}

}  // namespace qslc
