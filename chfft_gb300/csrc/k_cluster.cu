// Host side of the cluster latency form (k_cluster.cuh): the launch with a
// cluster-dimension attribute and the per-device function attributes.
#include "cluster.hpp"
#include "k_cluster.cuh"

namespace chfft {
namespace {

constexpr int kPasses = clus::kClusterMaxPasses;

template <typename T>
cudaError_t prepare(int csize, size_t smem) {
  // Function attributes are per device: set once per device and size.
  static int done_smem[64] = {0};
  static int done_np[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  auto fn = clus::k_c2c_cluster<T>;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (smem > 48 * 1024 && done_smem[dev] < (int)smem) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    done_smem[dev] = (int)smem;
  }
  if (csize > 8 && !done_np[dev]) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    done_np[dev] = 1;
  }
  return cudaSuccess;
}

template <typename T>
cudaError_t launch_t(const clus::ClusterArgs& a, long long batch, int csize, int threads, size_t smem,
                     cudaStream_t s) {
  cudaError_t e = prepare<T>(csize, smem);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)(batch * csize), 1, 1);
  cfg.blockDim = dim3((unsigned)threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)csize;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, clus::k_c2c_cluster<T>, a);
}

template <typename T>
int max_clusters_t(int csize, int threads, size_t smem) {
  if (prepare<T>(csize, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)csize, 1, 1);
  cfg.blockDim = dim3((unsigned)threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)csize;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, clus::k_c2c_cluster<T>, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

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

}  // namespace

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

cudaError_t cluster_launch(int dtype, const clus::ClusterArgs& a, long long batch, int csize, int threads,
                           size_t smem, cudaStream_t s) {
  return dtype == 0 ? launch_t<float>(a, batch, csize, threads, smem, s)
                    : launch_t<double>(a, batch, csize, threads, smem, s);
}

int cluster_max_active(int dtype, int csize, int threads, size_t smem) {
  return dtype == 0 ? max_clusters_t<float>(csize, threads, smem) : max_clusters_t<double>(csize, threads, smem);
}

}  // namespace chfft
