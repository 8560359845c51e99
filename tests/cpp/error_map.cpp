// How the C++ drop-in reports failures of the C ABI: builds
// qsl::Qubits<qsl::cuda_type, double>(n), applies one gate, reads prob and
// prints what happened -- "ok", or the exception type the reference's
// callers would catch and its message.  The failures come from the host:
// an impossible allocation, a machine without a GPU, or an entry point made
// to fail by QSLC_FORCE_ERROR.
//
// usage: error_map <nqubits>
#include <qsl/qubits/cuda.hpp>

#include <cstdio>
#include <cstdlib>
#include <stdexcept>

int main(int argc, char **argv)
{
    const unsigned n = argc > 1 ? unsigned(std::atoi(argv[1])) : 4;
    try {
        qsl::Qubits<qsl::cuda_type, double> q(n);
        q.rotateX(0, 0.3);
        const double p = q.prob(0, 1);
        std::printf("ok %.17g\n", p);
    } catch (const std::logic_error &e) {
        std::printf("logic_error: %s\n", e.what());
    } catch (const std::runtime_error &e) {
        std::printf("runtime_error: %s\n", e.what());
    }
    return 0;
}
