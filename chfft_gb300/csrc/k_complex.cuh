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
__global__ void __launch_bounds__(kMaxThreads, CoreT::kMinBlocks) k_c2c(const KArgs a) {
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
__global__ void __launch_bounds__(kMaxThreads, CoreT::kMinBlocks) k_cols(const KArgs a) {
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

// ---------------------------------------------------------------- four-step
// A length-N FFT with N = N1 * N2 beyond one CTA (x[n1 N2 + n2]):
//   pass A: column FFTs of length N1, times w_N^(k1 n2), in place layout;
//   pass B: row FFTs of length N2, written transposed to X[k1 + N1 k2].
// The inter-pass twiddle comes from two tables: w_N^e = hi[e / L] lo[e % L],
// L a power of two so the split is a shift and a mask
// (FourStep in kernels.cuh).

// Pass A loader: MODE 0 plain (scale, conjugate for backward); MODE 1 the
// Bluestein input x_j c_j for flat index j = n1 N2 + n2 < n_user, else 0.
template <typename C, int MODE>
struct ColsALoad {
  const C* in;  // first column of the tile
  int ncols, nvalid, c0;
  typename Real<C>::type scale;
  int back;
  const FourStep* fs;
  __device__ __forceinline__ C load(int t, int i) const {
    if (t >= nvalid) return czero<C>();
    if (MODE == 1) {
      const long long j = (long long)i * ncols + c0 + t;
      if (j >= fs->n_user) return czero<C>();
      C v = cscale(in[(long long)i * ncols + t], scale);
      if (back) v = cconj(v);
      return cmul(v, __ldg(&static_cast<const C*>(fs->chirp)[j]));
    }
    C v = cscale(in[(long long)i * ncols + t], scale);
    return back ? cconj(v) : v;
  }
};

template <typename C>
struct ColsAStore {
  C* out;
  int ncols, nvalid, c0;
  const FourStep* fs;
  __device__ __forceinline__ void store(int t, int k1, C v) const {
    if (t >= nvalid) return;
    const long long e = (long long)k1 * (c0 + t);  // < N
    const C* lo = static_cast<const C*>(fs->lo);
    const C* hi = static_cast<const C*>(fs->hi);
    const C w = cmul(__ldg(&hi[e >> fs->tw_shift]), __ldg(&lo[e & ((1LL << fs->tw_shift) - 1)]));
    out[(long long)k1 * ncols + t] = cmul(v, w);
  }
};

template <typename T, class CoreT, int MODE>
__global__ void __launch_bounds__(kMaxThreads, CoreT::kMinBlocks) k_cols_tw(const KArgs a, const FourStep fs) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const auto sm = CoreT::template tile<C>(smem_raw, a.ld);
  const long long tr = blockIdx.x / a.tiles_per_tr;
  const int c0 = (int)(blockIdx.x - tr * a.tiles_per_tr) * a.tpb;
  const int nvalid = min(a.tpb, a.ncols - c0);
  ColsALoad<C, MODE> ld{(const C*)a.in + tr * a.in_dist + c0, a.ncols, nvalid, c0, (T)a.scale, a.back, &fs};
  ColsAStore<C> st{(C*)a.out + tr * a.out_dist + c0, a.ncols, nvalid, c0, &fs};
  CoreT::run(a.core, a.tpb, sm, ld, st);
}

// Pass B storer, element k2 of row k1 goes to X[k1 + N1 k2]:
// MODE 0 plain (conjugate for backward, the pass-A scale already applied);
// MODE 1 Bluestein spectrum: conj(X_k B^_k), the inverse FFT's input;
// MODE 2 Bluestein output: k < n_user gets conj(X_k) c_k (conjugated again
// for backward).
template <typename C, int MODE>
struct RowsBStore {
  C* out;  // transform base
  int r0, nvalid, n1, back;
  const FourStep* fs;
  __device__ __forceinline__ void store(int t, int k2, C v) const {
    if (t >= nvalid) return;
    const long long k = (long long)(r0 + t) + (long long)n1 * k2;
    if (MODE == 0) {
      out[k] = back ? cconj(v) : v;
    } else if (MODE == 1) {
      out[k] = cconj(cmul(v, __ldg(&static_cast<const C*>(fs->bhat)[k])));
    } else {
      if (k < fs->n_user) {
        C y = cmul(cconj(v), __ldg(&static_cast<const C*>(fs->chirp)[k]));
        out[k] = back ? cconj(y) : y;
      }
    }
  }
};

template <typename C>
struct RowsBLoad {
  const C* in;  // first row of the tile
  int n2, nvalid;
  __device__ __forceinline__ C load(int t, int i) const {
    return t < nvalid ? in[(long long)t * n2 + i] : czero<C>();
  }
};

template <typename T, class CoreT, int MODE>
__global__ void __launch_bounds__(kMaxThreads, CoreT::kMinBlocks) k_rows_t(const KArgs a, const FourStep fs) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const auto sm = CoreT::template tile<C>(smem_raw, a.ld);
  const long long tr = blockIdx.x / a.tiles_per_tr;
  const int r0 = (int)(blockIdx.x - tr * a.tiles_per_tr) * a.tpb;
  const int nvalid = min(a.tpb, fs.n1 - r0);
  // Rows are contiguous: load them with consecutive threads along a row,
  // then run the FFT with consecutive threads across rows so the transposed
  // store is contiguous. Compile-time-stage cores fuse the row load into
  // their first pass; the others stage it through the tile.
  RowsBLoad<C> rl{(const C*)a.in + tr * a.in_dist + (long long)r0 * fs.n2, fs.n2, nvalid};
  RowsBStore<C, MODE> st{(C*)a.out + tr * a.out_dist, r0, nvalid, fs.n1, a.back, &fs};
  if constexpr (CoreT::kStatic) {
    CoreT::template run<true>(a.core, a.tpb, sm, rl, st);
  } else {
    load_phase<false>(sm, fs.n2, a.tpb, rl);
    CoreT::run(a.core, a.tpb, sm, sm, st);
  }
}

}  // namespace kern

#ifndef __CUDACC_RTC__
template <typename T>
cudaError_t launch_fourstep(bool pass_a, int mode, bool k1, const KArgs& a, const FourStep& fs,
                            unsigned blocks, unsigned threads, size_t smem, cudaStream_t stream) {
  using namespace kern;
  void (*fn)(const KArgs, const FourStep) = nullptr;
  if (pass_a) {
    using K1C = DynCore<false, true, true, true>;
    using KNC = DynCore<false, true, true, false>;
    if (mode == 0) fn = k1 ? k_cols_tw<T, K1C, 0> : k_cols_tw<T, KNC, 0>;
    else fn = k1 ? k_cols_tw<T, K1C, 1> : k_cols_tw<T, KNC, 1>;
  } else {
    using K1C = DynCore<false, true, true, true>;
    using KNC = DynCore<false, true, true, false>;
    if (mode == 0) fn = k1 ? k_rows_t<T, K1C, 0> : k_rows_t<T, KNC, 0>;
    else if (mode == 1) fn = k1 ? k_rows_t<T, K1C, 1> : k_rows_t<T, KNC, 1>;
    else fn = k1 ? k_rows_t<T, K1C, 2> : k_rows_t<T, KNC, 2>;
  }
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  fn<<<blocks, threads, smem, stream>>>(a, fs);
  return cudaGetLastError();
}

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
