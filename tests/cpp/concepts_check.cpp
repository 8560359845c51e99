// Compile-time proof of the drop-in: qsl's own concepts (concepts.hpp:51-126)
// accept the CUDA backends.  Built against qsl's headers where they exist
// (-DWITH_QSL_HEADERS), else against qsl/cuda_standalone.hpp.
#ifdef WITH_QSL_HEADERS
#include <qsl/qubits.hpp>
#endif
#include <qsl/qubits/cuda.hpp>

using CudaD = qsl::Qubits<qsl::cuda_type, double>;
using CudaF = qsl::Qubits<qsl::cuda_type, float>;
using CudaNPD = qsl::Qubits<qsl::cuda_np_type, double>;
using CudaNPF = qsl::Qubits<qsl::cuda_np_type, float>;
using CudaRD = qsl::Qubits<qsl::cuda_resize_type, double>;
using CudaRF = qsl::Qubits<qsl::cuda_resize_type, float>;

#ifdef WITH_QSL_HEADERS
static_assert(qsl::Simulator<CudaD> && qsl::Simulator<CudaF>);
static_assert(qsl::HasAllGates<CudaD> && qsl::HasAllGates<CudaF>);
static_assert(qsl::HasMeasurement<CudaD> && qsl::HasMeasurement<CudaF>);
static_assert(qsl::NPSimulator<CudaNPD> && qsl::NPSimulator<CudaNPF>);
static_assert(qsl::Simulator<CudaNPD>);
static_assert(!qsl::HasNonNPGates<CudaNPD>);
static_assert(qsl::Simulator<CudaRD> && qsl::Simulator<CudaRF>);
static_assert(qsl::HasAllGates<CudaRD> && qsl::HasMeasurement<CudaRF>);
// the members qsl's Resize backend adds (resize.hpp:160-180, :310, :350)
static_assert(std::is_same_v<decltype(std::declval<CudaRD &>().measureOut(0u)),
                             decltype(std::declval<qsl::Qubits<qsl::Type::Resize, double> &>().measureOut(0u))>);
static_assert(std::is_same_v<decltype(std::declval<CudaRF &>().postselectOut(0u, 0u)),
                             decltype(std::declval<qsl::Qubits<qsl::Type::Resize, float> &>().postselectOut(0u, 0u))>);
// qsl's gate member-pointer aliases (qubits.hpp:89-96) bind to our members
qsl::OneQubitGate<CudaD, double> g1 = &CudaD::rotateX;
qsl::TwoQubitGate<CudaD> g2 = &CudaD::controlNot;
qsl::TwoQubitGate<CudaNPD, double> g3 = &CudaNPD::npRotateX;
#endif
static_assert(std::is_copy_constructible_v<CudaD> && std::is_copy_assignable_v<CudaD>);
static_assert(std::is_copy_constructible_v<CudaRD> && std::is_copy_assignable_v<CudaRD>);
static_assert(requires(CudaRD q) { q.addQubit(0u); q.appendQubit(); q.reallocateState(); });
static_assert(std::is_same_v<CudaD::Fp_type, double> && std::is_same_v<CudaNPF::Fp_type, float>);

int main() { return 0; }
