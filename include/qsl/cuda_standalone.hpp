/*
 * cuda_standalone.hpp -- the few qsl declarations the CUDA backend needs,
 * for programs built without qsl's own headers.
 *
 * When qsl's include/qsl/qubits.hpp is included first, qsl/qubits/cuda.hpp
 * uses qsl's declarations instead and this file is not read.  The
 * declarations here have the same layout and names as qsl's:
 *   qsl::complex<Fp>  -- {Fp real; Fp imag;} (include/qsl/utils/complex.hpp:40-49)
 *   qsl::Type         -- the backend enum (include/qsl/qubits.hpp:57-63),
 *                        here with Cuda, CudaNP and CudaResize added
 *   qsl::Qubits       -- the primary template (include/qsl/qubits.hpp:75)
 */
#ifndef QSL_CUDA_STANDALONE_HPP
#define QSL_CUDA_STANDALONE_HPP

#include <concepts>
#include <ostream>

namespace qsl {

template <std::floating_point Fp = double>
struct complex {
    Fp real;
    Fp imag;
    complex(Fp r, Fp i) : real(r), imag(i) {}
    complex() : complex(0, 0) {}
};

enum class Type {
    Default,
    Omp,
    NP,
    OmpNP,
    Resize,
    Cuda = 0x100,     ///< GB300 state-vector backend (qsl/qubits/cuda.hpp)
    CudaNP = 0x101,   ///< GB300 number-preserving backend
    CudaResize = 0x102,   ///< GB300 resizeable backend
};

template <Type T = Type::Default, std::floating_point Fp = double>
class Qubits;

}  // namespace qsl

#endif
