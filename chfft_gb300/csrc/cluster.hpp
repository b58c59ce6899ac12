// Host interface of the cluster latency form (k_cluster.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace chfft {
namespace clus {
struct ClusterArgs;
}

// The kernel for a split: the compile-time-shape instance of (n1, n2,
// csize) when there is one (its thread count into *threads; CHFFT_CLUSTER_STATIC=0
// skips them), else the run-time-shape kernel (*threads unchanged).
const void* cluster_kernel(int dtype, int n1, int n2, int csize, int* threads);
// One launch of kernel fn: `batch` transforms, one cluster of `csize` CTAs (8 or 16) each.
cudaError_t cluster_launch(const void* fn, const clus::ClusterArgs& a, long long batch, int csize, int threads,
                           size_t smem, cudaStream_t s);
// Per-pass input twiddles of a cluster FFT of length n (pass radices in
// `code`, 4 bits each): rows 1 .. np - 1, n entries each, into out.
cudaError_t cluster_pass_tables(int dtype, int n, unsigned long long code, int np, void* out, cudaStream_t s);
// The four-step twiddles w_n^(n2 k1) x scale at n2 * n1 + k1.
cudaError_t cluster_block_table(int dtype, long long n, int n1, double scale, void* out, cudaStream_t s);
// RFft1D around a cluster FFT of the half length h (k_cluster.cu): the
// split of batch forward cores z (h complex each) into out (h + 1 each),
// times scale; the merge of batch inputs (h + 1 each) into z (h each),
// times s2, for a backward (conjugating) core. Programmatic dependent
// launches on s.
cudaError_t rfft_split(int dtype, const void* z, void* out, const void* coef, int h, long long batch, double scale,
                       cudaStream_t s);
cudaError_t rfft_merge(int dtype, const void* in, void* z, const void* bcoef, int h, long long batch, double s2,
                       cudaStream_t s);
// Dct1D / Mdct1D around a cluster FFT: op kDct2 / kDct3 (core N/2), kMdct /
// kImdct (core N/4, the forward FFT for both). real_pre turns batch inputs
// into the core's input z (scale and the DCT ortho factor applied as the
// one-CTA kernels do); real_post turns the core's output into the outputs
// (DCT-III's core runs backward; the MDCT scale applied here). n is the
// user length. Programmatic dependent launches on s.
enum { kDct2 = 0, kDct3 = 1, kMdct = 2, kImdct = 3 };
cudaError_t real_pre(int dtype, int op, const void* in, void* z, const void* aux0, const void* aux1, int n,
                     long long batch, double scale, double ortho, cudaStream_t s);
cudaError_t real_post(int dtype, int op, const void* z, void* out, const void* aux0, const void* aux1, int n,
                      long long batch, double scale, cudaStream_t s);
// Clusters of this shape the current device can hold at once (0: none, the
// shape cannot launch).
int cluster_max_active(const void* fn, int csize, int threads, size_t smem);

}  // namespace chfft
