// double instantiation of the real-data transform kernels (k_real.cuh).
#include "k_real.cuh"

namespace chfft {
template cudaError_t launch_real<double>(Kernel, bool, bool, const KArgs&, unsigned, unsigned, size_t, cudaStream_t);
}  // namespace chfft
