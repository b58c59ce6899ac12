// double instantiation of the four-step pass kernels (k_complex.cuh).
#include "k_complex.cuh"

namespace chfft {
template cudaError_t launch_fourstep<double>(bool, int, bool, const KArgs&, const FourStep&, unsigned, unsigned, size_t,
                                         cudaStream_t);
}  // namespace chfft
