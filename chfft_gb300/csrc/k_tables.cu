// Plan-time table generation on the GPU. Every entry is computed in FP64
// (CUDA's sincospi/sinpi on an exactly reduced rational argument) and then
// rounded once to the working dtype. chfft computes its tables in the
// working precision (src/precompute_utils.rs:15-68), so the f32 tables here
// are more accurate than the reference's; the chirp index k*k mod 2N is
// computed exactly in 64-bit integers like src/cfft1d.rs:123-128.
#include "kernels.cuh"

namespace chfft {

namespace {

template <typename C>
__device__ __forceinline__ void put(void* out, long long k, double re, double im) {
  using R = typename Real<C>::type;
  reinterpret_cast<C*>(out)[k] = mk(R(re), R(im));
}

// exp(-2 pi i p / q) for integers 0 <= p < q, with the numerator reduced to
// (-q/2, q/2] so the sincospi argument stays small and exact-ish.
__device__ __forceinline__ void root(long long p, long long q, double* c, double* s) {
  p %= q;
  if (2 * p > q) p -= q;
  sincospi(2.0 * (double)p / (double)q, s, c);
  *s = -*s;
}

template <typename T>
__global__ void k_gen(int which, long long n, long long count, long long m, void* out) {
  using C = cx_t<T>;
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  double c, s;
  switch ((Table)which) {
    case Table::OMEGA:
      root(k, n, &c, &s);
      put<C>(out, k, c, s);
      break;
    case Table::CHIRP: {
      const unsigned long long idx = ((unsigned long long)k * (unsigned long long)k) % (2ull * (unsigned long long)n);
      root((long long)idx, 2 * n, &c, &s);  // exp(-pi i idx / n)
      put<C>(out, k, c, s);
      break;
    }
    case Table::RCOEF:  // (1 + i w^k)/2, w^k = (c, s): i w^k = (-s, c)
      root(k, n, &c, &s);
      put<C>(out, k, 0.5 * (1.0 - s), 0.5 * c);
      break;
    case Table::RBCOEF:  // (1 - i w^-k)/2, w^-k = (c, -s): i w^-k = (s, c)
      root(k, n, &c, &s);
      put<C>(out, k, 0.5 * (1.0 - s), -0.5 * c);
      break;
    case Table::OMEGA4N_POS:
      root(k, 4 * n, &c, &s);
      put<C>(out, k, c, -s);
      break;
    case Table::OMEGA4N_NEG:
      root(k, 4 * n, &c, &s);
      put<C>(out, k, c, s);
      break;
    case Table::MDCT_TW: {
      root(8 * k + 1, 8 * n, &c, &s);
      const double sc = sqrt(sqrt(2.0 / (double)n));
      put<C>(out, k, c * sc, s * sc);
      break;
    }
    case Table::SINE_WIN:
      reinterpret_cast<T*>(out)[k] = (T)sinpi(((double)k + 0.5) / (double)n);
      break;
    case Table::VORBIS_WIN: {
      const double v = sinpi(((double)k + 0.5) / (double)n);
      reinterpret_cast<T*>(out)[k] = (T)sinpi(0.5 * v * v);
      break;
    }
    case Table::BLUE_B: {
      // b_j = conj(c_|j|) for |j| < n placed circularly in length m, x 1/m.
      long long j = k < n ? k : (k > m - n ? m - k : -1);
      if (j < 0) {
        put<double2>(out, k, 0.0, 0.0);
      } else {
        const unsigned long long idx = ((unsigned long long)j * (unsigned long long)j) % (2ull * (unsigned long long)n);
        root((long long)idx, 2 * n, &c, &s);
        put<double2>(out, k, c / (double)m, -s / (double)m);
      }
      break;
    }
    case Table::CHIRP_INDEX:
      reinterpret_cast<unsigned long long*>(out)[k] =
          ((unsigned long long)k * (unsigned long long)k) % (2ull * (unsigned long long)n);
      break;
    case Table::OMEGA_STRIDE:
      root((long long)(((unsigned long long)k * (unsigned long long)m) % (unsigned long long)n), n, &c, &s);
      put<C>(out, k, c, s);
      break;
  }
}

template <typename T>
__global__ void k_gen_stage(PassList pl, long long total, void* out) {
  using C = cx_t<T>;
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= total) return;
  long long off = 0, ns = 1;
  for (int p = 0; p < pl.npass; p++) {
    const long long r = pl.r[p], blk = (r - 1) * ns;
    if (k < off + blk) {
      const long long e = k - off, jm = e % ns, rr = e / ns + 1;
      double c, s;
      root(jm * rr, ns * r, &c, &s);
      put<C>(out, k, c, s);
      return;
    }
    off += blk;
    ns *= r;
  }
}

template <typename T>
__global__ void k_from_f64(const double2* src, void* dst, long long count) {
  using C = cx_t<T>;
  using R = typename Real<C>::type;
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < count) reinterpret_cast<C*>(dst)[k] = mk(R(src[k].x), R(src[k].y));
}

}  // namespace

template <typename T>
cudaError_t gen_table(Table which, long long n, long long count, long long m, void* out, cudaStream_t stream) {
  if (count <= 0) return cudaSuccess;
  const unsigned threads = 256;
  const unsigned blocks = (unsigned)((count + threads - 1) / threads);
  k_gen<T><<<blocks, threads, 0, stream>>>((int)which, n, count, m, out);
  return cudaGetLastError();
}

template <typename T>
cudaError_t gen_stage_table(const PassList& pl, void* out, cudaStream_t stream) {
  long long total = 1;
  for (int p = 0; p < pl.npass; p++) total *= pl.r[p];
  total -= 1;
  if (total <= 0) return cudaSuccess;
  const unsigned threads = 256;
  k_gen_stage<T><<<(unsigned)((total + threads - 1) / threads), threads, 0, stream>>>(pl, total, out);
  return cudaGetLastError();
}

template <typename T>
cudaError_t convert_from_f64(const double2* src, void* dst, long long count, cudaStream_t stream) {
  if (count <= 0) return cudaSuccess;
  const unsigned threads = 256;
  const unsigned blocks = (unsigned)((count + threads - 1) / threads);
  k_from_f64<T><<<blocks, threads, 0, stream>>>(src, dst, count);
  return cudaGetLastError();
}

template cudaError_t gen_table<float>(Table, long long, long long, long long, void*, cudaStream_t);
template cudaError_t gen_table<double>(Table, long long, long long, long long, void*, cudaStream_t);
template cudaError_t gen_stage_table<float>(const PassList&, void*, cudaStream_t);
template cudaError_t gen_stage_table<double>(const PassList&, void*, cudaStream_t);
template cudaError_t convert_from_f64<float>(const double2*, void*, long long, cudaStream_t);
template cudaError_t convert_from_f64<double>(const double2*, void*, long long, cudaStream_t);

}  // namespace chfft
