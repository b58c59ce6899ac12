// Host side of the cluster latency form (k_cluster.cuh): the kernel choice
// (a compile-time-shape instance for the power-of-two splits, else the
// run-time-shape kernel), the launch with a cluster-dimension attribute,
// the per-device function attributes and the plan-time tables.
#include <cstdlib>
#include <map>
#include <mutex>
#include <utility>

#include "cluster.hpp"
#include "k_cluster.cuh"
#include "k_real.cuh"

namespace chfft {
namespace {

constexpr int kPasses = clus::kClusterMaxPasses;

using ClusterFn = void (*)(const clus::ClusterArgs);

// Function attributes are per device: the dynamic shared-memory size and
// (clusters of more than 8 CTAs) the non-portable cluster size, set once
// per (kernel, device) and size.
cudaError_t prepare(const void* fn, int csize, size_t smem) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, std::pair<size_t, bool>> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> g(mu);
  auto& d = done[{fn, dev}];
  if (smem > 48 * 1024 && d.first < smem) {
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    d.first = smem;
  }
  if (csize > 8 && !d.second) {
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    d.second = true;
  }
  return cudaSuccess;
}

void cluster_config(cudaLaunchConfig_t* cfg, cudaLaunchAttribute* at, long long batch, int csize, int threads,
                    size_t smem, cudaStream_t s) {
  *cfg = cudaLaunchConfig_t{};
  cfg->gridDim = dim3((unsigned)(batch * csize), 1, 1);
  cfg->blockDim = dim3((unsigned)threads, 1, 1);
  cfg->dynamicSmemBytes = smem;
  cfg->stream = s;
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)csize;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  // Programmatic dependent launch: the kernels wait for their prerequisites
  // before reading the input (k_cluster.cuh), so this launch may begin
  // while the previous kernel on the stream finishes.
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[1].val.programmaticStreamSerializationAllowed = 1;
  cfg->attrs = at;
  cfg->numAttrs = 2;
}

struct StaticInst {
  int n1, n2, cs, threads;
  ClusterFn f32, f64;
};
#define CHFFT_CLUSTER_INST(A, B, CS)                                                                      \
  StaticInst {                                                                                          \
    A, B, CS, clus::CShape<A, B, CS>::THREADS, clus::k_c2c_cluster_s<float, A, B, CS>,                  \
        clus::k_c2c_cluster_s<double, A, B, CS>                                                         \
  }
// The splits the plans pick for N = 2^6 .. 2^14 (fewest passes, then the
// most balanced; 8 CTAs below 1024 points, 16 from there).
const StaticInst kStatic[] = {
    CHFFT_CLUSTER_INST(8, 8, 8),     CHFFT_CLUSTER_INST(8, 16, 8),    CHFFT_CLUSTER_INST(16, 16, 8),
    CHFFT_CLUSTER_INST(16, 32, 8),   CHFFT_CLUSTER_INST(16, 64, 16),  CHFFT_CLUSTER_INST(32, 64, 16),
    CHFFT_CLUSTER_INST(64, 64, 16),  CHFFT_CLUSTER_INST(64, 128, 16), CHFFT_CLUSTER_INST(128, 128, 16),
};
#undef CHFFT_CLUSTER_INST

// exp(-2 pi i e / n) in FP64 for 0 <= e < n, the numerator reduced to
// (-n/2, n/2] so the sincospi argument stays small.
__device__ __forceinline__ void root64(long long e, long long n, double* c, double* s) {
  e %= n;
  if (2 * e > n) e -= n;
  sincospi(2.0 * (double)e / (double)n, s, c);
  *s = -*s;
}

struct PassTab {
  int np;
  int r[kPasses], ns[kPasses];
};

// Row p - 1 (p = 1 .. np - 1) holds the input twiddle of pass p at input
// position i: r = i / (n / R_p), jm = (i mod (n / R_p)) mod Ns_p,
// w_n^(r jm n / (Ns_p R_p)). FP64, rounded once.
template <typename T>
__global__ void k_pass_tables(PassTab pt, int n, void* out) {
  using C = cx_t<T>;
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (long long)(pt.np - 1) * n) return;
  const int p = (int)(k / n) + 1, i = (int)(k % n);
  const int R = pt.r[p], Ns = pt.ns[p], nb = n / R;
  const int r = i / nb, jm = (i % nb) % Ns;
  double c, sn;
  root64((long long)r * jm * (n / (Ns * R)), n, &c, &sn);
  reinterpret_cast<C*>(out)[k] = mk((T)c, (T)sn);
}

// out[k] = w_n^((k / n1) (k mod n1)) x scale: the four-step twiddles in
// [n2][k1] order. FP64, rounded once.
template <typename T>
__global__ void k_block_table(long long n, int n1, double scale, void* out) {
  using C = cx_t<T>;
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double c, sn;
  root64((long long)(((unsigned long long)(k / n1) * (unsigned long long)(k % n1)) % (unsigned long long)n), n, &c,
         &sn);
  reinterpret_cast<C*>(out)[k] = mk((T)(c * scale), (T)(sn * scale));
}

// RFft1D around the cluster FFT of the half length h: the split after a
// forward core (src/rfft1d.rs:136-148: X_i = Z_i - x, X_{h-i} = Z_{h-i} +
// conj x, x = coef_i (Z_i - conj Z_{h-i}); DC, Nyquist and N/4 bins from
// item 0), times the method's scale; and the merge before a backward core
// (src/rfft1d.rs:132-145), times 2 scale (the core then runs the conjugated
// forward FFT). Thread (t, i < ceil(N/4)) of the grid. Launched after or
// before a cluster kernel with programmatic dependent launch: each waits for
// the kernels before it before reading.
template <typename T>
__global__ void k_rfft_split(const cx_t<T>* z, cx_t<T>* out, const cx_t<T>* coef, int h, long long batch, T scale) {
  using C = cx_t<T>;
  clus::allow_dependents();
  clus::wait_prerequisites();
  const int qlen = (2 * h + 3) >> 2;
  const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= batch * qlen) return;
  const long long t = w / qlen;
  const int i = (int)(w - t * qlen);
  const C* zt = z + t * h;
  C* o = out + t * (h + 1);
  if (i == 0) {
    const C z0 = zt[0];
    o[0] = mk((z0.x + z0.y) * scale, T(0));
    o[h] = mk((z0.x - z0.y) * scale, T(0));
    if (((2 * h) & 3) == 0) o[qlen] = cscale(cconj(zt[qlen]), scale);
  } else {
    const C zi = zt[i], zh = zt[h - i];
    const C x = cmul(coef[i], csub(zi, cconj(zh)));
    o[i] = cscale(csub(zi, x), scale);
    o[h - i] = cscale(cadd(zh, cconj(x)), scale);
  }
}

template <typename T>
__global__ void k_rfft_merge(const cx_t<T>* in, cx_t<T>* z, const cx_t<T>* bcoef, int h, long long batch, T s2) {
  using C = cx_t<T>;
  clus::allow_dependents();
  clus::wait_prerequisites();
  const int qlen = (2 * h + 3) >> 2;
  const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= batch * qlen) return;
  const long long t = w / qlen;
  const int i = (int)(w - t * qlen);
  const C* s = in + t * (h + 1);
  C* zt = z + t * h;
  if (i == 0) {
    const C s0 = s[0], sh = s[h];
    zt[0] = mk((s0.x + sh.x) * T(0.5) * s2, (s0.x - sh.x) * T(0.5) * s2);
    if (((2 * h) & 3) == 0) zt[qlen] = cscale(cconj(s[qlen]), s2);
  } else {
    const C si = s[i], sh = s[h - i];
    const C x = cmul(bcoef[i], csub(si, cconj(sh)));
    zt[i] = cscale(csub(si, x), s2);
    zt[h - i] = cscale(cadd(sh, cconj(x)), s2);
  }
}

// Dct1D and Mdct1D around a cluster FFT of the core length m (N/2, N/4):
// the pre- and post-processing of the one-CTA kernels (k_real.cuh), as
// their own launches on a workspace of m complex per transform. Pointwise
// steps reuse the kernels' loaders / storers; the paired ones (DCT-II's
// post-twiddle, DCT-III's merge) restate their loops on global memory.
template <typename T, class Ld>
__global__ void k_pre(Ld ld, cx_t<T>* z, int m, long long batch) {
  clus::allow_dependents();
  clus::wait_prerequisites();
  const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= batch * m) return;
  const long long t = w / m;
  z[w] = ld.load((int)t, (int)(w - t * m));
}

template <typename T, class St>
__global__ void k_post(St st, const cx_t<T>* z, int m, long long batch, int conj_in) {
  clus::allow_dependents();
  clus::wait_prerequisites();
  const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= batch * m) return;
  const long long t = w / m;
  const cx_t<T> v = z[w];
  st.store((int)t, (int)(w - t * m), conj_in ? cconj(v) : v);
}

// DCT-II post-twiddle with exp(+i pi k / 2N) (src/dct1d.rs:266-289) of the
// forward core output z (h per transform) into out (N reals each).
template <typename T>
__global__ void k_dct2_post(const cx_t<T>* zs, T* out, const cx_t<T>* coef, const cx_t<T>* om, int h,
                            long long batch) {
  using C = cx_t<T>;
  clus::allow_dependents();
  clus::wait_prerequisites();
  const int N = 2 * h, q2 = (N + 3) >> 2;
  const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= batch * q2) return;
  const long long t = w / q2;
  const int i = (int)(w - t * q2);
  const C* z = zs + t * h;
  T* o = out + t * N;
  if (i == 0) {
    const C z0 = z[0];
    o[0] = z0.x + z0.y;
    o[h] = (z0.x - z0.y) * om[h].x;
    if ((N & 3) == 0) {
      const C x = cmul(z[q2], om[q2]);
      o[q2] = x.x;
      o[N - q2] = x.y;
    }
  } else {
    const C zi = z[i];
    const C wconj = cconj(z[h - i]);
    const C x = cmul(coef[i], csub(zi, wconj));
    const C j = cmul(cconj(csub(zi, x)), om[i]);
    o[i] = j.x;
    o[N - i] = j.y;
    const C k = cmul(cadd(wconj, x), om[h - i]);
    o[h - i] = k.x;
    o[h + i] = k.y;
  }
}

// DCT-III pre-twiddle and merge (src/dct1d.rs:369-391) of the input (N reals
// per transform) into z (h each) for a backward (conjugating) core: the
// values the one-CTA kernel's tile holds, conjugated.
template <typename T>
__global__ void k_dct3_pre(const T* xs, cx_t<T>* zs, const cx_t<T>* coef, const cx_t<T>* om, int h, long long batch,
                           T scale, T ortho) {
  using C = cx_t<T>;
  clus::allow_dependents();
  clus::wait_prerequisites();
  const int N = 2 * h, q = (N + 3) >> 2;
  const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= batch * q) return;
  const long long t = w / q;
  const int i = (int)(w - t * q);
  const T* x = xs + t * N;
  C* z = zs + t * h;
  if (i == 0) {
    const T zval = x[0] * ortho, hval = x[h] * om[h].x;
    z[0] = mk((zval + hval) * scale, (zval - hval) * scale);
    if ((N & 3) == 0) z[q] = cmul(mk(x[q], x[N - q]), cscale(om[q], scale));
  } else {
    const C j = cconj(cscale(cmul(mk(x[i], x[N - i]), om[i]), scale));
    const C k = cscale(cmul(mk(x[h - i], x[h + i]), om[h - i]), scale);
    const C xx = cmul(coef[i], csub(j, k));
    z[i] = csub(j, xx);
    z[h - i] = cconj(cadd(k, xx));
  }
}

template <typename K, typename... Args>
cudaError_t pdl_launch(K kernel, unsigned blocks, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(blocks, 1, 1);
  cfg.blockDim = dim3(256, 1, 1);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

}  // namespace

cudaError_t rfft_split(int dtype, const void* z, void* out, const void* coef, int h, long long batch, double scale,
                       cudaStream_t s) {
  const long long items = batch * ((2LL * h + 3) >> 2);
  const unsigned blocks = (unsigned)((items + 255) / 256);
  if (dtype == 0)
    return pdl_launch(k_rfft_split<float>, blocks, s, static_cast<const float2*>(z), static_cast<float2*>(out),
                      static_cast<const float2*>(coef), h, batch, (float)scale);
  return pdl_launch(k_rfft_split<double>, blocks, s, static_cast<const double2*>(z), static_cast<double2*>(out),
                    static_cast<const double2*>(coef), h, batch, scale);
}

cudaError_t rfft_merge(int dtype, const void* in, void* z, const void* bcoef, int h, long long batch, double s2,
                       cudaStream_t s) {
  const long long items = batch * ((2LL * h + 3) >> 2);
  const unsigned blocks = (unsigned)((items + 255) / 256);
  if (dtype == 0)
    return pdl_launch(k_rfft_merge<float>, blocks, s, static_cast<const float2*>(in), static_cast<float2*>(z),
                      static_cast<const float2*>(bcoef), h, batch, (float)s2);
  return pdl_launch(k_rfft_merge<double>, blocks, s, static_cast<const double2*>(in), static_cast<double2*>(z),
                    static_cast<const double2*>(bcoef), h, batch, s2);
}

namespace {
unsigned blocks_for(long long items) { return (unsigned)((items + 255) / 256); }

template <typename T>
cudaError_t real_pre_t(int op, const void* in, void* z, const void* aux0, const void* aux1, int n, long long batch,
                       double scale, double ortho, cudaStream_t s) {
  using C = cx_t<T>;
  switch (op) {
    case kDct2: {
      const int h = n / 2;
      kern::DctPackLoad<T> ld{static_cast<const T*>(in), (long long)n, 0x7fffffff, n, (T)scale, (T)ortho};
      return pdl_launch(k_pre<T, kern::DctPackLoad<T>>, blocks_for(batch * h), s, ld, static_cast<C*>(z), h, batch);
    }
    case kDct3: {
      const int h = n / 2;
      return pdl_launch(k_dct3_pre<T>, blocks_for(batch * ((n + 3) >> 2)), s, static_cast<const T*>(in),
                        static_cast<C*>(z), static_cast<const C*>(aux0), static_cast<const C*>(aux1), h, batch,
                        (T)scale, (T)ortho);
    }
    case kMdct: {
      const int q = n / 4;
      kern::MdctLoad<T> ld{static_cast<const T*>(in), (long long)n, 0x7fffffff, n, static_cast<const C*>(aux0),
                           static_cast<const T*>(aux1)};
      return pdl_launch(k_pre<T, kern::MdctLoad<T>>, blocks_for(batch * q), s, ld, static_cast<C*>(z), q, batch);
    }
    default: {  // kImdct
      const int q = n / 4;
      kern::ImdctLoad<T> ld{static_cast<const T*>(in), (long long)(n / 2), 0x7fffffff, n / 2,
                            static_cast<const C*>(aux0)};
      return pdl_launch(k_pre<T, kern::ImdctLoad<T>>, blocks_for(batch * q), s, ld, static_cast<C*>(z), q, batch);
    }
  }
}

template <typename T>
cudaError_t real_post_t(int op, const void* z, void* out, const void* aux0, const void* aux1, int n, long long batch,
                        double scale, cudaStream_t s) {
  using C = cx_t<T>;
  switch (op) {
    case kDct2:
      return pdl_launch(k_dct2_post<T>, blocks_for(batch * ((n + 3) >> 2)), s, static_cast<const C*>(z),
                        static_cast<T*>(out), static_cast<const C*>(aux0), static_cast<const C*>(aux1), n / 2, batch);
    case kDct3: {
      kern::DctUnpackStore<T> st{static_cast<T*>(out), (long long)n, 0x7fffffff, n / 2};
      // the backward core's output is conj(v) of the one-CTA kernel's v
      return pdl_launch(k_post<T, kern::DctUnpackStore<T>>, blocks_for(batch * (n / 2)), s, st,
                        static_cast<const C*>(z), n / 2, batch, 1);
    }
    case kMdct: {
      kern::MdctStore<T> st{static_cast<T*>(out), (long long)(n / 2), 0x7fffffff, n / 2, static_cast<const C*>(aux0),
                            (T)scale};
      return pdl_launch(k_post<T, kern::MdctStore<T>>, blocks_for(batch * (n / 4)), s, st, static_cast<const C*>(z),
                        n / 4, batch, 0);
    }
    default: {  // kImdct
      kern::ImdctStore<T> st{static_cast<T*>(out), (long long)n, 0x7fffffff, n, static_cast<const C*>(aux0),
                             static_cast<const T*>(aux1), (T)scale};
      return pdl_launch(k_post<T, kern::ImdctStore<T>>, blocks_for(batch * (n / 4)), s, st, static_cast<const C*>(z),
                        n / 4, batch, 0);
    }
  }
}
}  // namespace

cudaError_t real_pre(int dtype, int op, const void* in, void* z, const void* aux0, const void* aux1, int n,
                     long long batch, double scale, double ortho, cudaStream_t s) {
  return dtype == 0 ? real_pre_t<float>(op, in, z, aux0, aux1, n, batch, scale, ortho, s)
                    : real_pre_t<double>(op, in, z, aux0, aux1, n, batch, scale, ortho, s);
}

cudaError_t real_post(int dtype, int op, const void* z, void* out, const void* aux0, const void* aux1, int n,
                      long long batch, double scale, cudaStream_t s) {
  return dtype == 0 ? real_post_t<float>(op, z, out, aux0, aux1, n, batch, scale, s)
                    : real_post_t<double>(op, z, out, aux0, aux1, n, batch, scale, s);
}

cudaError_t cluster_pass_tables(int dtype, int n, unsigned long long code, int np, void* out, cudaStream_t s) {
  PassTab pt{};
  pt.np = np;
  for (int p = 0, ns = 1; p < np; p++) {
    pt.r[p] = (int)((code >> (4 * p)) & 15);
    pt.ns[p] = ns;
    ns *= pt.r[p];
  }
  const long long total = (long long)(np - 1) * n;
  if (total <= 0) return cudaSuccess;
  const unsigned blocks = (unsigned)((total + 255) / 256);
  if (dtype == 0)
    k_pass_tables<float><<<blocks, 256, 0, s>>>(pt, n, out);
  else
    k_pass_tables<double><<<blocks, 256, 0, s>>>(pt, n, out);
  return cudaGetLastError();
}

cudaError_t cluster_block_table(int dtype, long long n, int n1, double scale, void* out, cudaStream_t s) {
  const unsigned blocks = (unsigned)((n + 255) / 256);
  if (dtype == 0)
    k_block_table<float><<<blocks, 256, 0, s>>>(n, n1, scale, out);
  else
    k_block_table<double><<<blocks, 256, 0, s>>>(n, n1, scale, out);
  return cudaGetLastError();
}

const void* cluster_kernel(int dtype, int n1, int n2, int csize, int* threads) {
  const char* e = std::getenv("CHFFT_CLUSTER_STATIC");
  if (!(e && e[0] == '0'))
    for (const auto& k : kStatic)
      if (k.n1 == n1 && k.n2 == n2 && k.cs == csize) {
        *threads = k.threads;
        return reinterpret_cast<const void*>(dtype == 0 ? k.f32 : k.f64);
      }
  return reinterpret_cast<const void*>(dtype == 0 ? clus::k_c2c_cluster<float> : clus::k_c2c_cluster<double>);
}

cudaError_t cluster_launch(const void* fn, const clus::ClusterArgs& a, long long batch, int csize, int threads,
                           size_t smem, cudaStream_t s) {
  cudaError_t e = prepare(fn, csize, smem);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg;
  cudaLaunchAttribute at[2];
  cluster_config(&cfg, at, batch, csize, threads, smem, s);
  return cudaLaunchKernelEx(&cfg, reinterpret_cast<ClusterFn>(const_cast<void*>(fn)), a);
}

int cluster_max_active(const void* fn, int csize, int threads, size_t smem) {
  if (prepare(fn, csize, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  cudaLaunchConfig_t cfg;
  cudaLaunchAttribute at[2];
  cluster_config(&cfg, at, 1, csize, threads, smem, nullptr);
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, fn, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

}  // namespace chfft
