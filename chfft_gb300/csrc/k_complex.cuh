// Complex-input kernels: batched C2C rows and column tiles (the second
// dimension of CFft2D), each with a mixed-radix or a fused Bluestein core.
// Each kernel is a template over a core policy (engine.cuh): k_complex_f32.cu
// / k_complex_f64.cu instantiate the run-time-stage kernels, the plan-time
// compiler (jit.cu) instantiates compile-time-stage ones.
#pragma once

#include "kernels.cuh"

namespace chfft {

namespace kern {

// ---------------------------------------------------------------- rows
// Contiguous sequences. The backward transform conjugates on the way in and
// out (conj(F(conj x)) = F^-1 x up to scale), so one set of forward
// twiddles serves both directions. The scale is applied on load, as chfft's
// out-of-place path does in its gather (src/mixed_radix.rs:32-43).
template <typename C>
struct RowLoad {
  const C* in;
  long long dist;
  int nvalid;
  typename Real<C>::type scale;
  int back;
  __device__ __forceinline__ C load(int t, int i) const {
    if (t >= nvalid) return czero<C>();
    C v = cscale(in[(long long)t * dist + i], scale);
    return back ? cconj(v) : v;
  }
};

template <typename C>
struct RowStore {
  C* out;
  long long dist;
  int nvalid;
  int back;
  __device__ __forceinline__ void store(int t, int i, C v) const {
    if (t < nvalid) out[(long long)t * dist + i] = back ? cconj(v) : v;
  }
};

template <typename T, class CoreT>
__global__ void __launch_bounds__(kMaxThreads, CoreT::kK1 ? 2 : 1) k_c2c(const KArgs a) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const auto sm = CoreT::template tile<C>(smem_raw, a.ld);
  const long long t0 = (long long)blockIdx.x * a.tpb;
  const int nvalid = (int)min((long long)a.tpb, a.count - t0);
  RowLoad<C> ld{(const C*)a.in + t0 * a.in_dist, a.in_dist, nvalid, (T)a.scale, a.back};
  RowStore<C> st{(C*)a.out + t0 * a.out_dist, a.out_dist, nvalid, a.back};
  CoreT::run(a.core, a.tpb, sm, ld, st);
}

// ---------------------------------------------------------------- columns
// Transform `count` arrays of core.n rows x ncols columns along the rows
// dimension (each column is one sequence with stride ncols). A CTA takes
// tpb adjacent columns, so every row segment it touches is contiguous; the
// TMINOR mapping makes consecutive threads walk adjacent columns.
template <typename C>
struct ColLoad {
  const C* in;  // first column of the tile
  int ncols, nvalid;
  typename Real<C>::type scale;
  int back;
  __device__ __forceinline__ C load(int t, int i) const {
    if (t >= nvalid) return czero<C>();
    C v = cscale(in[(long long)i * ncols + t], scale);
    return back ? cconj(v) : v;
  }
};

template <typename C>
struct ColStore {
  C* out;
  int ncols, nvalid, back;
  __device__ __forceinline__ void store(int t, int i, C v) const {
    if (t < nvalid) out[(long long)i * ncols + t] = back ? cconj(v) : v;
  }
};

template <typename T, class CoreT>
__global__ void __launch_bounds__(kMaxThreads, CoreT::kK1 ? 2 : 1) k_cols(const KArgs a) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const auto sm = CoreT::template tile<C>(smem_raw, a.ld);
  const long long tr = blockIdx.x / a.tiles_per_tr;
  const int c0 = (int)(blockIdx.x - tr * a.tiles_per_tr) * a.tpb;
  const int nvalid = min(a.tpb, a.ncols - c0);
  ColLoad<C> ld{(const C*)a.in + tr * a.in_dist + c0, a.ncols, nvalid, (T)a.scale, a.back};
  ColStore<C> st{(C*)a.out + tr * a.out_dist + c0, a.ncols, nvalid, a.back};
  CoreT::run(a.core, a.tpb, sm, ld, st);
}

}  // namespace kern

#ifndef __CUDACC_RTC__
template <typename T>
cudaError_t launch_complex(Kernel which, bool blue, bool k1, const KArgs& a, unsigned blocks, unsigned threads,
                           size_t smem, cudaStream_t stream) {
  using namespace kern;
  void (*fn)(const KArgs) = nullptr;
#define CHFFT_PICK(K, TMINOR)                                                                  \
  (blue ? (k1 ? K<T, DynCore<true, TMINOR, true, true>> : K<T, DynCore<true, TMINOR, true, false>>) \
        : (k1 ? K<T, DynCore<false, TMINOR, true, true>> : K<T, DynCore<false, TMINOR, true, false>>))
  switch (which) {
    case Kernel::C2C: fn = CHFFT_PICK(k_c2c, false); break;
    case Kernel::COLS: fn = CHFFT_PICK(k_cols, true); break;
    default: return cudaErrorInvalidValue;
  }
#undef CHFFT_PICK
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  fn<<<blocks, threads, smem, stream>>>(a);
  return cudaGetLastError();
}
#endif  // __CUDACC_RTC__

}  // namespace chfft
