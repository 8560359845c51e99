// qsl's own cross-checking framework, qsl::Verify with its checkers
// (include/qsl/verify.hpp:65-140, include/qsl/verify/checkers.hpp:223-1282),
// instantiated with the CUDA backends as the second simulator, the way qsl's
// basic tests pair Default with Omp, NP and Resize
// (src/tests/basic-tests.cpp:406-560).  Every checker's member calls
// (copy-construction, setState/getState, measure, postselect, sample,
// sampleAll, prob and every gate through a member pointer) are therefore
// instantiated against the drop-in.
//
// Built only where qsl's headers exist, linked against qsl's own Default/NP
// implementation and libqslc.  Run with a GPU:  verify_check [nqubits nones]
// exits 0 when every checker agrees within the bounds qsl's basic tests use.
#include <qsl/qubits.hpp>
#include <qsl/verify.hpp>
#include <qsl/qubits/cuda.hpp>

#include <cmath>
#include <cstdio>
#include <cstdlib>

namespace {

int failures = 0;

void expect(bool ok, const char *what)
{
    if (!ok) {
        std::fprintf(stderr, "FAILED: %s\n", what);
        ++failures;
    }
}

// The statistics every measurement checker reports, with the bounds of
// src/tests/basic-tests.cpp:425-458.
template <typename V>
void measurement_checks(V &verify, double state_tol)
{
    auto prob = verify.template check<qsl::ProbChecker>();
    expect(std::abs(prob.template mean<double>(1)) < 1e-10, "prob outcome 0 difference");
    expect(std::abs(prob.template mean<double>(2)) < 1e-10, "prob outcome 1 difference");

    auto meas = verify.template check<qsl::MeasureChecker>();
    expect(std::abs(meas.template mean<double>(1) - 1) < 1e-10, "measure interval overlap");

    auto post = verify.template check<qsl::PostselectChecker>();
    expect(std::abs(post.template mean<double>(1)) < 1e-10, "postselect prob 0");
    expect(std::abs(post.template mean<double>(2)) < 1e-10, "postselect prob 1");
    expect(std::abs(post.template mean<double>(3)) < state_tol, "postselect state 0");
    expect(std::abs(post.template mean<double>(4)) < state_tol, "postselect state 1");

    auto sample = verify.template check<qsl::SampleChecker>();
    expect(std::abs(sample.template mean<double>(1) - 1) < 1e-10, "sample interval overlap");

    auto all = verify.template check<qsl::SampleAllChecker>();
    expect(std::abs(all.overlap_rate - 1) < 1e-10, "sampleAll interval overlap");
    expect(std::abs(all.mean_relative_error) < 0.15, "sampleAll relative error");
}

template <typename Table>
void gate_checks(const Table &gates)
{
    for (const auto &[gate, table] : gates) {
        expect(std::abs(table.template mean<double>("distance")) < 1e-9, gate.c_str());
    }
}

} // namespace

int main(int argc, char **argv)
{
    const unsigned nqubits = argc > 1 ? std::atoi(argv[1]) : 8;
    const unsigned nones = argc > 2 ? std::atoi(argv[2]) : 5;

    using Default = qsl::Qubits<qsl::Type::Default, double>;
    using NP = qsl::Qubits<qsl::Type::NP, double>;
    using Cuda = qsl::Qubits<qsl::cuda_type, double>;
    using CudaNP = qsl::Qubits<qsl::cuda_np_type, double>;
    using Resize = qsl::Qubits<qsl::Type::Resize, double>;
    using CudaResize = qsl::Qubits<qsl::cuda_resize_type, double>;

    qsl::Verify<Default, Cuda, qsl::DefaultStateGen<double>, qsl::MeasureChecker,
                qsl::PostselectChecker, qsl::SampleChecker, qsl::SampleAllChecker,
                qsl::ProbChecker, qsl::DefaultGateChecker>
        full;
    full.configureState(nqubits);
    full.configureChecker<qsl::SampleAllChecker>(1000000, 0.99);
    measurement_checks(full, 1e-7);
    gate_checks(full.check<qsl::DefaultGateChecker>());

    qsl::Verify<NP, CudaNP, qsl::NPStateGen<double>, qsl::MeasureChecker,
                qsl::PostselectChecker, qsl::SampleChecker, qsl::SampleAllChecker,
                qsl::ProbChecker, qsl::NPGateChecker>
        np;
    np.configureState(nqubits, nones);
    np.configureChecker<qsl::SampleAllChecker>(1000000, 0.99);
    measurement_checks(np, 1e-10);
    gate_checks(np.check<qsl::NPGateChecker>());

    qsl::Verify<Resize, CudaResize, qsl::DefaultStateGen<double>, qsl::MeasureChecker,
                qsl::PostselectChecker, qsl::SampleChecker, qsl::SampleAllChecker,
                qsl::ProbChecker, qsl::DefaultGateChecker>
        resize;
    resize.configureState(nqubits);
    resize.configureChecker<qsl::SampleAllChecker>(1000000, 0.99);
    measurement_checks(resize, 1e-10);
    gate_checks(resize.check<qsl::DefaultGateChecker>());

    std::printf("%s: %d failed checks\n", failures ? "FAIL" : "OK", failures);
    return failures ? 1 : 0;
}
