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
__global__ void __launch_bounds__(CoreT::kThreads, CoreT::kMinBlocks) k_c2c(const KArgs a) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const auto sm = CoreT::template tile<C>(smem_raw, a.ld);
  const long long t0 = (long long)blockIdx.x * a.tpb;
  const int nvalid = (int)min((long long)a.tpb, a.count - t0);
  RowLoad<C> ld{(const C*)a.in + t0 * a.in_dist, a.in_dist, nvalid, (T)a.scale, a.back};
  RowStore<C> st{(C*)a.out + t0 * a.out_dist, a.out_dist, nvalid, a.back};
  CoreT::run(a.core, a.tpb, sm, ld, st);
}

// ---------------------------------------------------------------- rows, split complex
// The same rows with real and imaginary parts in separate arrays (a native
// layout the reference does not offer; chfft takes interleaved
// Complex<T>, src/cfft1d.rs:270). KArgs: in / aux0 the input's real /
// imaginary parts, out / aux1 the output's.
template <typename C>
struct SplitLoad {
  using R = typename Real<C>::type;
  const R* re;
  const R* im;
  long long dist;
  int nvalid;
  R scale;
  int back;
  __device__ __forceinline__ C load(int t, int i) const {
    if (t >= nvalid) return czero<C>();
    const long long k = (long long)t * dist + i;
    const C v = mk(re[k] * scale, im[k] * scale);
    return back ? cconj(v) : v;
  }
};

template <typename C>
struct SplitStore {
  using R = typename Real<C>::type;
  R* re;
  R* im;
  long long dist;
  int nvalid;
  int back;
  __device__ __forceinline__ void store(int t, int i, C v) const {
    if (t >= nvalid) return;
    const long long k = (long long)t * dist + i;
    re[k] = v.x;
    im[k] = back ? -v.y : v.y;
  }
};

template <typename T, class CoreT>
__global__ void __launch_bounds__(CoreT::kThreads, CoreT::kMinBlocks) k_c2c_split(const KArgs a) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const auto sm = CoreT::template tile<C>(smem_raw, a.ld);
  const long long t0 = (long long)blockIdx.x * a.tpb;
  const int nvalid = (int)min((long long)a.tpb, a.count - t0);
  SplitLoad<C> ld{(const T*)a.in + t0 * a.in_dist, (const T*)a.aux0 + t0 * a.in_dist, a.in_dist, nvalid, (T)a.scale,
                  a.back};
  SplitStore<C> st{(T*)a.out + t0 * a.out_dist, (T*)const_cast<void*>(a.aux1) + t0 * a.out_dist, a.out_dist, nvalid,
                   a.back};
  CoreT::run(a.core, a.tpb, sm, ld, st);
}

// ---------------------------------------------------------------- rows, strided
// Element i of transform t at t * dist + i * stride (complex elements), for
// input and output separately (a native layout beyond the reference's
// contiguous slices: matrix columns, padded rows, interleaved channels).
// KArgs: in_dist / out_dist the distances, ncols / n_user the input /
// output strides.
template <typename C>
struct StridedLoad {
  const C* in;
  long long dist, stride;
  int nvalid;
  typename Real<C>::type scale;
  int back;
  __device__ __forceinline__ C load(int t, int i) const {
    if (t >= nvalid) return czero<C>();
    const C v = cscale(in[(long long)t * dist + (long long)i * stride], scale);
    return back ? cconj(v) : v;
  }
};

template <typename C>
struct StridedStore {
  C* out;
  long long dist, stride;
  int nvalid;
  int back;
  __device__ __forceinline__ void store(int t, int i, C v) const {
    if (t < nvalid) out[(long long)t * dist + (long long)i * stride] = back ? cconj(v) : v;
  }
};

template <typename T, class CoreT>
__global__ void __launch_bounds__(CoreT::kThreads, CoreT::kMinBlocks) k_c2c_strided(const KArgs a) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const auto sm = CoreT::template tile<C>(smem_raw, a.ld);
  const long long t0 = (long long)blockIdx.x * a.tpb;
  const int nvalid = (int)min((long long)a.tpb, a.count - t0);
  StridedLoad<C> ld{(const C*)a.in + t0 * a.in_dist, a.in_dist, (long long)a.ncols, nvalid, (T)a.scale, a.back};
  StridedStore<C> st{(C*)a.out + t0 * a.out_dist, a.out_dist, (long long)a.n_user, nvalid, a.back};
  CoreT::run(a.core, a.tpb, sm, ld, st);
}

// ---------------------------------------------------------------- rows, Rader
// A prime length N whose N - 1 = L is 7-smooth (N = 1009: L = 2^4 3^2 7)
// by Rader's algorithm instead of Chirp-Z (src/chirpz.rs:87-146 computes
// the same DFT with two FFTs of M = 2048). With g a primitive root mod N,
//   X_0 = x_0 + sum_p a_p,   X_{g^-q} = x_0 + (a (*) b)_q,
//   a_p = x_{g^p},  b_m = w_N^(g^-m),  (*) the cyclic convolution of length L,
// so the core runs two L-point FFTs: FFT_L(a), times B^ = FFT_L(b) / L
// (conjugated: the inverse runs as a forward FFT), FFT_L again. The rows are
// staged contiguously in shared memory (buffer R, stride ldr); the first
// FFT's first pass gathers a_p = R[g^p], its last pass stores the spectrum
// product and keeps X_0 = x_0 + A_0; the second FFT's last pass scatters
// x_0 + C_q to R[g^-q]; a contiguous store phase writes the rows out.
// KArgs: aux0 = the permutations (L ints g^p mod N, then L ints g^-q mod N),
// aux1 = B^ (L values), n_user = N, ncols = ldr; core = the L-point core.
template <typename C>
struct RaderGather {
  const C* r;
  int ldr;
  const int* perm;  // g^p mod N
  __device__ __forceinline__ C load(int t, int p) const { return r[t * ldr + __ldg(&perm[p])]; }
};

template <typename C, class Tile>
struct RaderSpectrum {
  const Tile& sm;
  const C* bhat;  // FFT_L(b) / L
  const C* r;
  int ldr;
  C* x0;          // per sequence: X_0 = x_0 + A_0
  __device__ __forceinline__ void store(int t, int k, C v) const {
    if (k == 0) x0[t] = cadd(r[t * ldr], v);
    sm.store(t, k, cconj(cmul(v, __ldg(&bhat[k]))));
  }
};

template <typename C>
struct RaderScatter {
  C* r;
  int ldr;
  const int* perm;  // g^-q mod N (never 0, so x_0 = R[0] stays readable)
  __device__ __forceinline__ void store(int t, int q, C v) const {
    r[t * ldr + __ldg(&perm[q])] = cadd(r[t * ldr], cconj(v));
  }
};

template <typename T, class CoreT>
__global__ void __launch_bounds__(CoreT::kThreads, CoreT::kMinBlocks) k_c2c_rader(const KArgs a) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const auto sm = CoreT::template tile<C>(smem_raw, a.ld);
  const int L = a.core.n, N = a.n_user, ldr = a.ncols;
  C* r = reinterpret_cast<C*>(smem_raw + (((size_t)a.tpb * a.ld * sizeof(C) + 15) / 16) * 16);
  C* x0 = r + (size_t)a.tpb * ldr;
  const long long t0 = (long long)blockIdx.x * a.tpb;
  const int nvalid = (int)min((long long)a.tpb, a.count - t0);
  const C* in = (const C*)a.in + t0 * a.in_dist;
  // Stage the rows, kU loads in flight per thread before their stores.
  constexpr int kU = 8;
  const int total = a.tpb * N;
  for (int b0 = threadIdx.x; b0 < total; b0 += kU * blockDim.x) {
    C v[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const int b = b0 + u * blockDim.x, t = b / N, i = b - t * N;
      v[u] = czero<C>();
      if (b < total && t < nvalid) v[u] = in[(long long)t * a.in_dist + i];
    }
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const int b = b0 + u * blockDim.x, t = b / N, i = b - t * N;
      if (b < total) {
        const C w = cscale(v[u], (T)a.scale);
        r[t * ldr + i] = a.back ? cconj(w) : w;
      }
    }
  }
  __syncthreads();
  const int* perm = static_cast<const int*>(a.aux0);
  RaderGather<C> gather{r, ldr, perm};
  RaderSpectrum<C, decltype(sm)> spec{sm, static_cast<const C*>(a.aux1), r, ldr, x0};
  CoreT::run(a.core, a.tpb, sm, gather, spec);
  RaderScatter<C> scatter{r, ldr, perm + L};
  CoreT::run(a.core, a.tpb, sm, sm, scatter);
  __syncthreads();
  C* out = (C*)a.out + t0 * a.out_dist;
  for (int b = threadIdx.x; b < nvalid * N; b += blockDim.x) {
    const int t = b / N, i = b - t * N;
    const C v = i == 0 ? x0[t] : r[t * ldr + i];
    out[(long long)t * a.out_dist + i] = a.back ? cconj(v) : v;
  }
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
__global__ void __launch_bounds__(CoreT::kThreads, CoreT::kMinBlocks) k_cols(const KArgs a) {
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

// The four-step kernels' MODE template argument: bits 0-1 the pass mode;
// bit 3 (kSmemTwiddle): pass A builds, per CTA, the tables
// A[t][q] = w_N^(32 q c) and B[t][r] = w_N^(r c) (c = c0 + t, q < ceil(N1 / 32),
// r < 32) in shared memory after its tile, so the store's w_N^(k1 c) =
// A[t][k1 / 32] B[t][k1 % 32] costs two shared loads instead of two global
// table loads per element.
constexpr int kSmemTwiddle = 8;

// Pass A loader: MODE 0 plain (scale, conjugate for backward); MODE 1 the
// Bluestein input x_j c_j for flat index j = n1 N2 + n2 < n_user, else 0.
template <typename C, int MODE>
struct ColsALoad {
  const C* in;  // first column of the tile
  int ncols, nvalid, c0;
  typename Real<C>::type scale;
  int back;
  const FourStep* fs;
  __device__ __forceinline__ C get(long long k) const { return in[k]; }
  __device__ __forceinline__ C load(int t, int i) const {
    if (t >= nvalid) return czero<C>();
    if (MODE == 1) {
      const long long j = (long long)i * ncols + c0 + t;
      if (j >= fs->n_user) return czero<C>();
      C v = cscale(get((long long)i * ncols + t), scale);
      if (back) v = cconj(v);
      return cmul(v, __ldg(&static_cast<const C*>(fs->chirp)[j]));
    }
    C v = cscale(get((long long)i * ncols + t), scale);
    return back ? cconj(v) : v;
  }
};

template <typename C, bool STWID = false>
struct ColsAStore {
  C* out;
  int ncols, nvalid, c0;
  const FourStep* fs;
  const C* tw;             // STWID: the per-CTA tables A (tpb x qa) then B (tpb x qb), rows padded
  int qa, qb, tpb;
  __device__ __forceinline__ void store(int t, int k1, C v) const {
    if (t >= nvalid) return;
    C w;
    if constexpr (STWID) {
      w = cmul(tw[t * qa + (k1 >> 5)], tw[tpb * qa + t * qb + (k1 & 31)]);
    } else {
      const long long e = (long long)k1 * (c0 + t);  // < N
      const C* lo = static_cast<const C*>(fs->lo);
      const C* hi = static_cast<const C*>(fs->hi);
      w = cmul(__ldg(&hi[e >> fs->tw_shift]), __ldg(&lo[e & ((1LL << fs->tw_shift) - 1)]));
    }
    out[(long long)k1 * ncols + t] = cmul(v, w);
  }
};

// One pass-A tile: columns [c0, c0 + tpb) of transform tr_in of a.in,
// written to slot tr_out of a.out.
template <typename T, class CoreT, int MODE>
__device__ __forceinline__ void cols_tw_tile(const KArgs& a, const FourStep& fs, long long tr_in, long long tr_out,
                                             int c0, unsigned char* smem_raw) {
  using C = cx_t<T>;
  const auto sm = CoreT::template tile<C>(smem_raw, a.ld);
  const int nvalid = min(a.tpb, a.ncols - c0);
  ColsALoad<C, MODE & 3> ld{(const C*)a.in + tr_in * a.in_dist + c0, a.ncols, nvalid, c0, (T)a.scale, a.back,
                            &fs};
  constexpr bool kStw = (MODE & kSmemTwiddle) != 0;
  C* twt = nullptr;
  const int qa = smem_twiddle_stride_a(fs.n1), qb = smem_twiddle_stride_b(a.tpb);
  if constexpr (kStw) {
    // Tables after the tile (16-byte aligned); the core's first barrier
    // orders these writes before the last pass reads them.
    twt = reinterpret_cast<C*>(smem_raw + (((size_t)a.tpb * a.ld * sizeof(C) + 15) / 16) * 16);
    const C* lo = static_cast<const C*>(fs.lo);
    const C* hi = static_cast<const C*>(fs.hi);
    const long long mask = (1LL << fs.tw_shift) - 1;
    for (int i = threadIdx.x; i < a.tpb * (qa + qb); i += blockDim.x) {
      const bool in_a = i < a.tpb * qa;
      const int t = in_a ? i / qa : (i - a.tpb * qa) / qb;
      const int q = in_a ? i - t * qa : (i - a.tpb * qa) - t * qb;
      const long long e = ((long long)(in_a ? 32 * q : q) * (c0 + t)) % fs.n;  // w_N^N = 1
      twt[i] = cmul(__ldg(&hi[e >> fs.tw_shift]), __ldg(&lo[e & mask]));
    }
  }
  ColsAStore<C, kStw> st{(C*)a.out + tr_out * a.out_dist + c0, a.ncols, nvalid, c0, &fs, twt, qa, qb, a.tpb};
  CoreT::run(a.core, a.tpb, sm, ld, st);
}

template <typename T, class CoreT, int MODE>
__global__ void __launch_bounds__(CoreT::kThreads, CoreT::kMinBlocks) k_cols_tw(const KArgs a, const FourStep fs) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const long long tr = blockIdx.x / a.tiles_per_tr;
  const int c0 = (int)(blockIdx.x - tr * a.tiles_per_tr) * a.tpb;
  cols_tw_tile<T, CoreT, MODE>(a, fs, tr, tr, c0, smem_raw);
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
  __device__ __forceinline__ void put(long long k, C v) const { out[k] = v; }
  __device__ __forceinline__ void store(int t, int k2, C v) const {
    if (t >= nvalid) return;
    const long long k = (long long)(r0 + t) + (long long)n1 * k2;
    if (MODE == 0) {
      put(k, back ? cconj(v) : v);
    } else if (MODE == 1) {
      put(k, cconj(cmul(v, __ldg(&static_cast<const C*>(fs->bhat)[k]))));
    } else {
      if (k < fs->n_user) {
        C y = cmul(cconj(v), __ldg(&static_cast<const C*>(fs->chirp)[k]));
        put(k, back ? cconj(y) : y);
      }
    }
  }
};

template <typename C>
struct RowsBLoad {
  const C* in;  // first row of the tile
  int n2, nvalid;
  __device__ __forceinline__ C load(int t, int i) const {
    if (t >= nvalid) return czero<C>();
    return in[(long long)t * n2 + i];
  }
};

// One pass-B tile: rows [r0, r0 + tpb) of slot tr_in of a.in, transposed
// into transform tr_out of a.out.
template <typename T, class CoreT, int MODE>
__device__ __forceinline__ void rows_t_tile(const KArgs& a, const FourStep& fs, long long tr_in, long long tr_out,
                                            int r0, unsigned char* smem_raw) {
  using C = cx_t<T>;
  const auto sm = CoreT::template tile<C>(smem_raw, a.ld);
  const int nvalid = min(a.tpb, fs.n1 - r0);
  // Rows are contiguous: load them with consecutive threads along a row,
  // then run the FFT with consecutive threads across rows so the transposed
  // store is contiguous. Compile-time-stage cores fuse the row load into
  // their first pass; the others stage it through the tile.
  RowsBLoad<C> rl{(const C*)a.in + tr_in * a.in_dist + (long long)r0 * fs.n2, fs.n2, nvalid};
  RowsBStore<C, MODE & 3> st{(C*)a.out + tr_out * a.out_dist, r0, nvalid, fs.n1, a.back, &fs};
  if constexpr (CoreT::kStatic) {
    CoreT::template run<true>(a.core, a.tpb, sm, rl, st);
  } else {
    load_phase<false>(sm, fs.n2, a.tpb, rl);
    CoreT::run(a.core, a.tpb, sm, sm, st);
  }
}

template <typename T, class CoreT, int MODE>
__global__ void __launch_bounds__(CoreT::kThreads, CoreT::kMinBlocks) k_rows_t(const KArgs a, const FourStep fs) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const long long tr = blockIdx.x / a.tiles_per_tr;
  const int r0 = (int)(blockIdx.x - tr * a.tiles_per_tr) * a.tpb;
  rows_t_tile<T, CoreT, MODE>(a, fs, tr, tr, r0, smem_raw);
}

// ---------------------------------------------------------------- four-step Bluestein
// Middle pass of a four-step Bluestein transform (three passes instead of
// four). Rows k1 of pass A's output (n2 long): their FFT gives X at the
// natural index k = k1 + n1 k2; the inverse transform's input is
// conj(X_k B^_k) (the conjugation trick). The inverse FFT of length
// M = n1 n2 is split the other way round, m = m2 + n2 m1, so its first pass
// is again an n2-point FFT over k2 of the same row, followed by the twiddle
// w_M^(k1 m2); the row tile therefore runs two FFTs back to back and stores
// the intermediate as the n2 x n1 matrix [m2][k1] (contiguous runs of
// adjacent k1). The last pass is k_rows_t's chirp-out mode over the rows of
// that matrix (n1 and n2 swapped in its FourStep).
template <typename C, class Tile>
struct RowSpectrumStore {
  const Tile& sm;
  const C* bhat;
  int r0, n1;
  __device__ __forceinline__ void store(int t, int k2, C v) const {
    const int k1 = min(r0 + t, n1 - 1);  // rows past n1 are never stored
    sm.store(t, k2, cconj(cmul(v, __ldg(&bhat[k1 + (long long)n1 * k2]))));
  }
};

template <typename C>
struct RowsBBStore {
  C* out;  // the transform's n2 x n1 intermediate
  int r0, nvalid, n1;
  const FourStep* fs;
  __device__ __forceinline__ void store(int t, int m2, C v) const {
    if (t >= nvalid) return;
    const int k1 = r0 + t;
    const long long e = (long long)k1 * m2;  // < M
    const C* lo = static_cast<const C*>(fs->lo);
    const C* hi = static_cast<const C*>(fs->hi);
    const C w = cmul(__ldg(&hi[e >> fs->tw_shift]), __ldg(&lo[e & ((1LL << fs->tw_shift) - 1)]));
    const long long k = k1 + (long long)n1 * m2;
    out[k] = cmul(v, w);
  }
};

template <typename T, class CoreT, int MODE>
__global__ void __launch_bounds__(CoreT::kThreads, CoreT::kMinBlocks) k_rows_bb(const KArgs a, const FourStep fs) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const auto sm = CoreT::template tile<C>(smem_raw, a.ld);
  const long long tr = blockIdx.x / a.tiles_per_tr;
  const int r0 = (int)(blockIdx.x - tr * a.tiles_per_tr) * a.tpb;
  const int nvalid = min(a.tpb, fs.n1 - r0);
  RowsBLoad<C> rl{(const C*)a.in + tr * a.in_dist + (long long)r0 * fs.n2, fs.n2, nvalid};
  RowSpectrumStore<C, decltype(sm)> spec{sm, static_cast<const C*>(fs.bhat), r0, fs.n1};
  RowsBBStore<C> st{(C*)a.out + tr * a.out_dist, r0, nvalid, fs.n1, &fs};
  if constexpr (CoreT::kStatic) {
    CoreT::template run<true>(a.core, a.tpb, sm, rl, spec);
    CoreT::template run<false>(a.core, a.tpb, sm, sm, st);
  } else {
    load_phase<false>(sm, fs.n2, a.tpb, rl);
    CoreT::run(a.core, a.tpb, sm, sm, spec);
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
    else if (mode == 2) fn = k1 ? k_rows_t<T, K1C, 2> : k_rows_t<T, KNC, 2>;
    else fn = k1 ? k_rows_bb<T, K1C, 0> : k_rows_bb<T, KNC, 0>;  // 3: Bluestein middle pass
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
    case Kernel::C2C_SPLIT: fn = CHFFT_PICK(k_c2c_split, false); break;
    case Kernel::C2C_STRIDED: fn = CHFFT_PICK(k_c2c_strided, false); break;
    case Kernel::C2C_RADER:
      fn = k1 ? k_c2c_rader<T, DynCore<false, false, true, true>> : k_c2c_rader<T, DynCore<false, false, true, false>>;
      break;
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
