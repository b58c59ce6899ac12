// float instantiation of the row / column kernels (k_complex.cuh).
#include "k_complex.cuh"

namespace chfft {
template cudaError_t launch_complex<float>(Kernel, bool, bool, const KArgs&, unsigned, unsigned, size_t, cudaStream_t);
}  // namespace chfft
