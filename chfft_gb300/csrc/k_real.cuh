// Real-data transforms built on a shorter complex FFT, with their pre- and
// post-passes fused into the FFT kernel:
//   RFft1D   N reals <-> N/2+1 bins through an N/2 C2C (src/rfft1d.rs:115-187)
//   Dct1D    DCT-II / DCT-III through an N/2 C2C      (src/dct1d.rs:236-409)
//   Mdct1D   MDCT N -> N/2 / IMDCT N/2 -> N through an N/4 C2C
//            (src/mdct1d.rs:197-291)
// Pre-passes that need one input element per FFT input live in the first
// pass's loader and post-passes that need one FFT output per result live in
// the last pass's storer. Split steps that pair bin k with bin h-k run as a
// separate cooperative phase on the shared-memory tile.
// Run-time-stage instances come from k_real_f32.cu / k_real_f64.cu, plan-time
// specialised ones from jit.cu.
#pragma once

#include "kernels.cuh"

namespace chfft {

namespace kern {

struct BlockRange {
  long long t0;
  int nvalid;
};
__device__ __forceinline__ BlockRange block_range(const KArgs& a) {
  long long t0 = (long long)blockIdx.x * a.tpb;
  return {t0, (int)min((long long)a.tpb, a.count - t0)};
}

// ---------------------------------------------------------------- R2C
// z_m = (x_2m, x_2m+1) * scale (src/rfft1d.rs:128-131), read as one vector.
template <typename T>
struct PackLoad {
  using C = cx_t<T>;
  const T* in;
  long long dist;
  int nvalid;
  T scale;
  __device__ __forceinline__ C load(int t, int m) const {
    if (t >= nvalid) return czero<C>();
    return cscale(reinterpret_cast<const C*>(in + (long long)t * dist)[m], scale);
  }
};

template <typename T, class CoreT>
__global__ void __launch_bounds__(CoreT::kThreads, CoreT::kMinBlocks) k_r2c(const KArgs a) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const auto sm = CoreT::template tile<C>(smem_raw, a.ld);
  const BlockRange br = block_range(a);
  const int h = a.core.n, N = 2 * h;
  PackLoad<T> ld{(const T*)a.in + br.t0 * a.in_dist, a.in_dist, br.nvalid, (T)a.scale};
  CoreT::run(a.core, a.tpb,sm, ld, sm);
  // Split (src/rfft1d.rs:136-148): X_i = Z_i - x, X_{h-i} = Z_{h-i} + conj(x),
  // x = coef_i (Z_i - conj Z_{h-i}); DC / Nyquist / N/4 bins from item 0.
  const int qlen = (N + 3) >> 2;
  const C* coef = (const C*)a.aux0;
  for (int w = threadIdx.x; w < a.tpb * qlen; w += blockDim.x) {
    const int t = w / qlen, i = w - t * qlen;
    if (t >= br.nvalid) continue;
    C* o = (C*)a.out + (br.t0 + t) * a.out_dist;
    if (i == 0) {
      C z0 = sm.load(t, 0);
      o[0] = mk(z0.x + z0.y, T(0));
      o[h] = mk(z0.x - z0.y, T(0));
      if ((N & 3) == 0) o[qlen] = cconj(sm.load(t, qlen));
    } else {
      C zi = sm.load(t, i), zh = sm.load(t, h - i);
      C x = cmul(__ldg(&coef[i]), csub(zi, cconj(zh)));
      o[i] = csub(zi, x);
      o[h - i] = cadd(zh, cconj(x));
    }
  }
}

// ---------------------------------------------------------------- C2R
// Merge (src/rfft1d.rs:132-145) into the tile, inverse N/2 FFT, unpack
// re/im pairs x 2*scale (src/rfft1d.rs:129, :149-153).
template <typename T>
struct UnpackStore {
  using C = cx_t<T>;
  T* out;
  long long dist;
  int nvalid;
  T s2;
  __device__ __forceinline__ void store(int t, int m, C v) const {
    if (t < nvalid) reinterpret_cast<C*>(out + (long long)t * dist)[m] = mk(v.x * s2, -v.y * s2);
  }
};

template <typename T, class CoreT>
__global__ void __launch_bounds__(CoreT::kThreads, CoreT::kMinBlocks) k_c2r(const KArgs a) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const auto sm = CoreT::template tile<C>(smem_raw, a.ld);
  const BlockRange br = block_range(a);
  const int h = a.core.n, N = 2 * h;
  const int qlen = (N + 3) >> 2;
  const C* bcoef = (const C*)a.aux0;
  for (int w = threadIdx.x; w < a.tpb * qlen; w += blockDim.x) {
    const int t = w / qlen, i = w - t * qlen;
    if (t >= br.nvalid) continue;
    const C* s = (const C*)a.in + (br.t0 + t) * a.in_dist;
    if (i == 0) {
      C s0 = s[0], sh = s[h];
      sm.store(t, 0, mk((s0.x + sh.x) * T(0.5), -((s0.x - sh.x) * T(0.5))));
      if ((N & 3) == 0) sm.store(t, qlen, s[qlen]);  // conj(conj(s_q))
    } else {
      C si = s[i], sh = s[h - i];
      C x = cmul(__ldg(&bcoef[i]), csub(si, cconj(sh)));
      sm.store(t, i, cconj(csub(si, x)));
      sm.store(t, h - i, cconj(cadd(sh, cconj(x))));
    }
  }
  __syncthreads();
  UnpackStore<T> st{(T*)a.out + br.t0 * a.out_dist, a.out_dist, br.nvalid, T(2.0 * a.scale)};
  CoreT::run(a.core, a.tpb,sm, sm, st);
}

// ---------------------------------------------------------------- DCT-II
// Input reorder v = (x0, x2, ..., x_{N-2}, x_{N-1}, ..., x3, x1) packed as
// z_m = (v_2m, v_2m+1) * scale, x0 times the ortho factor
// (src/dct1d.rs:248-263).
template <typename T>
struct DctPackLoad {
  using C = cx_t<T>;
  const T* in;
  long long dist;
  int nvalid, n;
  T scale, ortho;
  __device__ __forceinline__ T v(const T* x, int j) const {
    return j < (n >> 1) ? x[2 * j] : x[2 * (n - 1 - j) + 1];
  }
  __device__ __forceinline__ C load(int t, int m) const {
    if (t >= nvalid) return czero<C>();
    const T* x = in + (long long)t * dist;
    T re = v(x, 2 * m), im = v(x, 2 * m + 1);
    if (m == 0) re *= ortho;
    return mk(re * scale, im * scale);
  }
};

template <typename T, class CoreT>
__global__ void __launch_bounds__(CoreT::kThreads, CoreT::kMinBlocks) k_dct2(const KArgs a) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const auto sm = CoreT::template tile<C>(smem_raw, a.ld);
  const BlockRange br = block_range(a);
  const int h = a.core.n, N = 2 * h;
  DctPackLoad<T> ld{(const T*)a.in + br.t0 * a.in_dist, a.in_dist, br.nvalid, N, (T)a.scale, (T)a.aux_scalar};
  CoreT::run(a.core, a.tpb,sm, ld, sm);
  // Post-twiddle with exp(+i pi k / 2N) (src/dct1d.rs:266-289).
  const int q2 = (N + 3) >> 2;
  const C* coef = (const C*)a.aux0;
  const C* om = (const C*)a.aux1;
  for (int w = threadIdx.x; w < a.tpb * q2; w += blockDim.x) {
    const int t = w / q2, i = w - t * q2;
    if (t >= br.nvalid) continue;
    T* o = (T*)a.out + (br.t0 + t) * a.out_dist;
    if (i == 0) {
      C z0 = sm.load(t, 0);
      o[0] = z0.x + z0.y;
      o[h] = (z0.x - z0.y) * __ldg(&om[h]).x;
      if ((N & 3) == 0) {
        C x = cmul(sm.load(t, q2), __ldg(&om[q2]));
        o[q2] = x.x;
        o[N - q2] = x.y;
      }
    } else {
      C zi = sm.load(t, i);
      C wconj = cconj(sm.load(t, h - i));
      C x = cmul(__ldg(&coef[i]), csub(zi, wconj));
      C j = cmul(cconj(csub(zi, x)), __ldg(&om[i]));
      o[i] = j.x;
      o[N - i] = j.y;
      C k = cmul(cadd(wconj, x), __ldg(&om[h - i]));
      o[h - i] = k.x;
      o[h + i] = k.y;
    }
  }
}

// ---------------------------------------------------------------- DCT-III
// Pre-twiddle and merge (src/dct1d.rs:369-391) into the tile, inverse N/2
// FFT, interleave out (src/dct1d.rs:395-408) from the last pass.
template <typename T>
struct DctUnpackStore {
  using C = cx_t<T>;
  T* out;
  long long dist;
  int nvalid, h;
  __device__ __forceinline__ void store(int t, int m, C v) const {
    if (t >= nvalid) return;
    T* o = out + (long long)t * dist;
    const T re = v.x, im = -v.y;  // conj(v)
    const int q = h >> 1;
    if (m < q) {
      o[4 * m] = re;
      o[4 * m + 2] = im;
    } else if ((h & 1) && m == q) {
      o[2 * h - 2] = re;
      o[2 * h - 1] = im;
    } else {
      const int i = h - 1 - m;
      o[4 * i + 1] = im;
      o[4 * i + 3] = re;
    }
  }
};

template <typename T, class CoreT>
__global__ void __launch_bounds__(CoreT::kThreads, CoreT::kMinBlocks) k_dct3(const KArgs a) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const auto sm = CoreT::template tile<C>(smem_raw, a.ld);
  const BlockRange br = block_range(a);
  const int h = a.core.n, N = 2 * h;
  const int q = (N + 3) >> 2;
  const C* coef = (const C*)a.aux0;
  const C* om = (const C*)a.aux1;
  const T scale = (T)a.scale, ortho = (T)a.aux_scalar;
  for (int w = threadIdx.x; w < a.tpb * q; w += blockDim.x) {
    const int t = w / q, i = w - t * q;
    if (t >= br.nvalid) continue;
    const T* x = (const T*)a.in + (br.t0 + t) * a.in_dist;
    if (i == 0) {
      T zval = x[0] * ortho;
      T hval = x[h] * __ldg(&om[h]).x;
      sm.store(t, 0, mk((zval + hval) * scale, -((zval - hval) * scale)));
      if ((N & 3) == 0) sm.store(t, q, cconj(cmul(mk(x[q], x[N - q]), cscale(__ldg(&om[q]), scale))));
    } else {
      C j = cconj(cscale(cmul(mk(x[i], x[N - i]), __ldg(&om[i])), scale));
      C k = cscale(cmul(mk(x[h - i], x[h + i]), __ldg(&om[h - i])), scale);
      C xx = cmul(__ldg(&coef[i]), csub(j, k));
      sm.store(t, i, cconj(csub(j, xx)));
      sm.store(t, h - i, cadd(k, xx));  // conj(conj(k) + conj(xx))
    }
  }
  __syncthreads();
  DctUnpackStore<T> st{(T*)a.out + br.t0 * a.out_dist, a.out_dist, br.nvalid, h};
  CoreT::run(a.core, a.tpb,sm, sm, st);
}

// ---------------------------------------------------------------- MDCT
// Window, fold and pre-twiddle (src/mdct1d.rs:206-230) as the loader of an
// N/4 FFT; post-twiddle (src/mdct1d.rs:232-241) as its storer.
struct MdctGeom {
  int lenh, lenq, leno, len3q, len5q;
  __device__ __forceinline__ explicit MdctGeom(int n) {
    lenh = n >> 1;
    lenq = lenh >> 1;
    leno = lenq - (lenq >> 1);
    len3q = lenh + lenq;
    len5q = lenh + len3q;
  }
};

template <typename T>
struct MdctLoad {
  using C = cx_t<T>;
  const T* in;
  long long dist;
  int nvalid, n;
  const C* tw;
  const T* win;
  __device__ __forceinline__ C load(int t, int i) const {
    if (t >= nvalid) return czero<C>();
    const T* x = in + (long long)t * dist;
    const MdctGeom g(n);
    const int k = i << 1;
    T re, im;
    if (i < g.leno) {
      re = x[g.len3q - 1 - k] * __ldg(&win[g.len3q - 1 - k]) + x[g.len3q + k] * __ldg(&win[g.len3q + k]);
      im = x[g.lenq + k] * __ldg(&win[g.lenq + k]) - x[g.lenq - 1 - k] * __ldg(&win[g.lenq - 1 - k]);
    } else {
      re = x[g.len3q - 1 - k] * __ldg(&win[g.len3q - 1 - k]) - x[k - g.lenq] * __ldg(&win[k - g.lenq]);
      im = x[g.lenq + k] * __ldg(&win[g.lenq + k]) + x[g.len5q - 1 - k] * __ldg(&win[g.len5q - 1 - k]);
    }
    return cmul(mk(re, im), __ldg(&tw[i]));
  }
};

template <typename T>
struct MdctStore {
  using C = cx_t<T>;
  T* out;
  long long dist;
  int nvalid, lenh;
  const C* tw;
  T scale;
  __device__ __forceinline__ void store(int t, int i, C v) const {
    if (t >= nvalid) return;
    T* o = out + (long long)t * dist;
    C r = cmul(v, cscale(__ldg(&tw[i]), scale));
    o[2 * i] = -r.x;
    o[lenh - 1 - 2 * i] = r.y;
  }
};

template <typename T, class CoreT>
__global__ void __launch_bounds__(CoreT::kThreads, CoreT::kMinBlocks) k_mdct(const KArgs a) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const auto sm = CoreT::template tile<C>(smem_raw, a.ld);
  const BlockRange br = block_range(a);
  const int n = a.n_user;
  const C* tw = (const C*)a.aux0;
  MdctLoad<T> ld{(const T*)a.in + br.t0 * a.in_dist, a.in_dist, br.nvalid, n, tw, (const T*)a.aux1};
  MdctStore<T> st{(T*)a.out + br.t0 * a.out_dist, a.out_dist, br.nvalid, n >> 1, tw, (T)a.scale};
  CoreT::run(a.core, a.tpb,sm, ld, st);
}

// IMDCT: pre-twiddle x(-2) (src/mdct1d.rs:259-263), FORWARD N/4 FFT, then
// post-twiddle, unfold and window (src/mdct1d.rs:268-289).
template <typename T>
struct ImdctLoad {
  using C = cx_t<T>;
  const T* in;
  long long dist;
  int nvalid, lenh;
  const C* tw;
  __device__ __forceinline__ C load(int t, int i) const {
    if (t >= nvalid) return czero<C>();
    const T* s = in + (long long)t * dist;
    return cmul(mk(s[2 * i], s[lenh - 1 - 2 * i]), cscale(__ldg(&tw[i]), T(-2.0)));
  }
};

template <typename T>
struct ImdctStore {
  using C = cx_t<T>;
  T* out;
  long long dist;
  int nvalid, n;
  const C* tw;
  const T* win;
  T scale;
  __device__ __forceinline__ void store(int t, int i, C v) const {
    if (t >= nvalid) return;
    T* o = out + (long long)t * dist;
    const MdctGeom g(n);
    const int k = i << 1;
    C r = cmul(v, cscale(__ldg(&tw[i]), scale));
    if (i < g.leno) {
      o[g.len3q - 1 - k] = r.x * __ldg(&win[g.len3q - 1 - k]);
      o[g.len3q + k] = r.x * __ldg(&win[g.len3q + k]);
      o[g.lenq + k] = -r.y * __ldg(&win[g.lenq + k]);
      o[g.lenq - 1 - k] = r.y * __ldg(&win[g.lenq - 1 - k]);
    } else {
      o[g.len3q - 1 - k] = r.x * __ldg(&win[g.len3q - 1 - k]);
      o[k - g.lenq] = -r.x * __ldg(&win[k - g.lenq]);
      o[g.lenq + k] = -r.y * __ldg(&win[g.lenq + k]);
      o[g.len5q - 1 - k] = -r.y * __ldg(&win[g.len5q - 1 - k]);
    }
  }
};

template <typename T, class CoreT>
__global__ void __launch_bounds__(CoreT::kThreads, CoreT::kMinBlocks) k_imdct(const KArgs a) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const auto sm = CoreT::template tile<C>(smem_raw, a.ld);
  const BlockRange br = block_range(a);
  const int n = a.n_user;
  const C* tw = (const C*)a.aux0;
  ImdctLoad<T> ld{(const T*)a.in + br.t0 * a.in_dist, a.in_dist, br.nvalid, n >> 1, tw};
  ImdctStore<T> st{(T*)a.out + br.t0 * a.out_dist, a.out_dist, br.nvalid, n, tw, (const T*)a.aux1, (T)a.scale};
  CoreT::run(a.core, a.tpb,sm, ld, st);
}

}  // namespace kern

#ifndef __CUDACC_RTC__
template <typename T>
cudaError_t launch_real(Kernel which, bool blue, bool k1, const KArgs& a, unsigned blocks, unsigned threads,
                        size_t smem, cudaStream_t stream) {
  void (*fn)(const KArgs) = nullptr;
  using namespace kern;
#define CHFFT_PICK(K)                                                                        \
  (blue ? (k1 ? K<T, DynCore<true, false, false, true>> : K<T, DynCore<true, false, false, false>>) \
        : (k1 ? K<T, DynCore<false, false, false, true>> : K<T, DynCore<false, false, false, false>>))
  switch (which) {
    case Kernel::R2C: fn = CHFFT_PICK(k_r2c); break;
    case Kernel::C2R: fn = CHFFT_PICK(k_c2r); break;
    case Kernel::DCT2: fn = CHFFT_PICK(k_dct2); break;
    case Kernel::DCT3: fn = CHFFT_PICK(k_dct3); break;
    case Kernel::MDCT: fn = CHFFT_PICK(k_mdct); break;
    case Kernel::IMDCT: fn = CHFFT_PICK(k_imdct); break;
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
