// Host side of the pipelined four-step launch (k_pipe.cuh): the tensor map
// over the input, the pass-A tiles' twiddle tables, the shape dispatch and
// the launch itself.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "k_pipe.cuh"
#include "pipe.hpp"

namespace chfft {
namespace {

typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
  static std::once_flag once;
  static EncodeTiled fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

template <int N1, int N2, bool BACK>
cudaError_t launch_dir(const pipe::TensorMap& tm, const pipe::PipeArgs& a, int grid, cudaStream_t s) {
  using S = pipe::Shape<N1, N2>;
  static_assert(S::SMEM <= 227 * 1024, "pipelined four-step tile does not fit shared memory");
  auto fn = pipe::k_pipe<N1, N2, BACK>;
  // The shared-memory attribute is a property of the function on the
  // current device: set once per device.
  static int done[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !done[dev]) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM);
    if (e != cudaSuccess) return e;
    done[dev] = 1;
  }
  fn<<<grid, pipe::kThreads, S::SMEM, s>>>(tm, a);
  return cudaGetLastError();
}

template <int N1, int N2>
cudaError_t launch_shape(const pipe::TensorMap& tm, const pipe::PipeArgs& a, int grid, cudaStream_t s) {
  return a.back ? launch_dir<N1, N2, true>(tm, a, grid, s) : launch_dir<N1, N2, false>(tm, a, grid, s);
}

// exp(-2 pi i e / n) in FP64 for 0 <= e < n, numerator reduced to (-n/2, n/2].
__device__ __forceinline__ float2 root_f32(long long e, long long n) {
  if (2 * e > n) e -= n;
  double c, sn;
  sincospi(2.0 * (double)e / (double)n, &sn, &c);
  return make_float2((float)c, (float)-sn);
}

// The pass-A tiles' twiddle tables (k_pipe.cuh): for tile q (columns
// c = q wa + t), atab[r][t] = w_N^(c r0 r) for r < 32, then
// wtab[j][t] = w_N^(c j) for j < r0 (r0 = n1 / 32), each computed in FP64
// and rounded once.
__global__ void k_pipe_twiddles(int n1, int n2, long long total, float2* out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int wa = pipe::kTileElems / n1, r0 = n1 / 32, per = (32 + r0) * wa;
  const long long n = (long long)n1 * n2;
  const long long q = i / per;
  const int e = (int)(i - q * per);
  const int row = e / wa, t = e - row * wa;
  const long long c = q * wa + t;
  const long long ex = row < 32 ? (c * r0 * row) % n : (c * (row - 32)) % n;
  out[i] = root_f32(ex, n);
}

}  // namespace

bool pipe_shape_ok(int n1, int n2) {
  auto ok = [](int v) { return v == 256 || v == 512 || v == 1024; };
  return ok(n1) && ok(n2);
}

size_t pipe_smem(int n1, int n2) {
#define CHFFT_PIPE_SMEM(A, B) \
  if (n1 == A && n2 == B) return pipe::Shape<A, B>::SMEM;
  CHFFT_PIPE_SMEM(256, 256) CHFFT_PIPE_SMEM(256, 512) CHFFT_PIPE_SMEM(256, 1024)
  CHFFT_PIPE_SMEM(512, 256) CHFFT_PIPE_SMEM(512, 512) CHFFT_PIPE_SMEM(512, 1024)
  CHFFT_PIPE_SMEM(1024, 256) CHFFT_PIPE_SMEM(1024, 512) CHFFT_PIPE_SMEM(1024, 1024)
#undef CHFFT_PIPE_SMEM
  return 0;
}

int pipe_tiles(int n1, int n2, int* ta, int* tb) {
  if (!pipe_shape_ok(n1, n2)) return 0;
  *ta = n2 / (pipe::kTileElems / n1);
  *tb = n1 / (pipe::kTileElems / n2);
  return 1;
}

size_t pipe_twiddle_elems(int n1, int n2) {
  if (!pipe_shape_ok(n1, n2)) return 0;
  const int wa = pipe::kTileElems / n1;
  return (size_t)(n2 / wa) * (size_t)((32 + n1 / 32) * wa);
}

cudaError_t pipe_twiddles(int n1, int n2, void* out, cudaStream_t s) {
  const long long total = (long long)pipe_twiddle_elems(n1, n2);
  if (total == 0) return cudaErrorInvalidValue;
  k_pipe_twiddles<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(n1, n2, total, static_cast<float2*>(out));
  return cudaGetLastError();
}

// Returns 0 on success, 1 when the input cannot be described by a tensor
// map (alignment) or the encoder is missing, 2 on a launch error.
int pipe_launch(int n1, int n2, const void* in, const pipe::PipeArgs& a, int grid, cudaStream_t s) {
  if (!pipe_shape_ok(n1, n2) || a.count <= 0 || grid <= 0) return 1;
  EncodeTiled enc = encoder();
  if (!enc || (reinterpret_cast<uintptr_t>(in) & 15)) return 1;
  const int wa = pipe::kTileElems / n1;
  pipe::TensorMap tm{};
  // The batch as a (count * n1) x n2 matrix of 8-byte complex elements;
  // boxes of wa columns x min(n1, 256) rows.
  const cuuint64_t dims[2] = {(cuuint64_t)n2, (cuuint64_t)a.count * (cuuint64_t)n1};
  const cuuint64_t strides[1] = {(cuuint64_t)n2 * 8};
  const cuuint32_t box[2] = {(cuuint32_t)wa, (cuuint32_t)(n1 < 256 ? n1 : 256)};
  const cuuint32_t estr[2] = {1, 1};
  static_assert(sizeof(pipe::TensorMap) == sizeof(CUtensorMap), "tensor map size");
  if (enc(reinterpret_cast<CUtensorMap*>(&tm), CU_TENSOR_MAP_DATA_TYPE_INT64, 2, const_cast<void*>(in), dims, strides,
          box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return 1;
  cudaError_t e = cudaErrorInvalidValue;
#define CHFFT_PIPE_LAUNCH(A, B) \
  if (n1 == A && n2 == B) e = launch_shape<A, B>(tm, a, grid, s);
  CHFFT_PIPE_LAUNCH(256, 256) CHFFT_PIPE_LAUNCH(256, 512) CHFFT_PIPE_LAUNCH(256, 1024)
  CHFFT_PIPE_LAUNCH(512, 256) CHFFT_PIPE_LAUNCH(512, 512) CHFFT_PIPE_LAUNCH(512, 1024)
  CHFFT_PIPE_LAUNCH(1024, 256) CHFFT_PIPE_LAUNCH(1024, 512) CHFFT_PIPE_LAUNCH(1024, 1024)
#undef CHFFT_PIPE_LAUNCH
  return e == cudaSuccess ? 0 : 2;
}

}  // namespace chfft
