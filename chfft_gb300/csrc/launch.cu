// Kernel dispatch by family (complex rows / columns, real-data kinds).
#include "kernels.cuh"

namespace chfft {

template <typename T>
cudaError_t launch_kernel(Kernel which, bool blue, bool k1, const KArgs& a, unsigned blocks, unsigned threads,
                          size_t smem, cudaStream_t stream) {
  if (which == Kernel::C2C || which == Kernel::COLS || which == Kernel::C2C_RADER || which == Kernel::C2C_SPLIT ||
      which == Kernel::C2C_STRIDED)
    return launch_complex<T>(which, blue, k1, a, blocks, threads, smem, stream);
  return launch_real<T>(which, blue, k1, a, blocks, threads, smem, stream);
}

template cudaError_t launch_kernel<float>(Kernel, bool, bool, const KArgs&, unsigned, unsigned, size_t, cudaStream_t);
template cudaError_t launch_kernel<double>(Kernel, bool, bool, const KArgs&, unsigned, unsigned, size_t, cudaStream_t);

}  // namespace chfft
