// Kernel argument block and host-callable launchers shared by the kernel
// translation units and the host plan code.
#pragma once

#ifndef __CUDACC_RTC__
#include <cuda_runtime.h>
#endif

#include "engine.cuh"

namespace chfft {

// One argument block for every transform kernel. Fields a kernel does not
// use stay zero. Element counts are in complex elements unless noted.
struct KArgs {
  CoreDesc core;           // complex core FFT (mixed radix or Bluestein)
  int tpb;                 // sequences (or columns) per CTA
  int ld;                  // shared-memory stride per sequence
  int back;                // 1: backward transform (conjugation trick)
  long long count;         // transforms in the batch
  long long tiles_per_tr;  // CTAs per transform (column kernels)
  const void* in;
  void* out;
  double scale;            // user scale factor (rounded to the working dtype)
  long long in_dist;       // elements between consecutive transforms (input)
  long long out_dist;      // elements between consecutive transforms (output)
  int ncols;               // column kernels: row length (distance between rows)
  int n_user;              // real transform length (MDCT)
  const void* aux0;        // kind tables (coef, twiddle)
  const void* aux1;        // second table (omega_4N, window)
  double aux_scalar;       // kind constant (DCT ortho factor)
  int* err;                // device error word, may be null
};

enum class Kernel : int {
  C2C = 0,
  COLS = 1,
  R2C = 2,
  C2R = 3,
  DCT2 = 4,
  DCT3 = 5,
  MDCT = 6,
  IMDCT = 7,
  COLS_TW = 8,  // four-step pass A
  ROWS_T = 9,   // four-step pass B
  ROWS_BB = 10, // four-step Bluestein middle pass (k_rows_bb)
  C2C_RADER = 11, // rows of a prime length by Rader's algorithm (k_c2c_rader)
  C2C_SPLIT = 12, // rows with separate real / imaginary arrays (k_c2c_split, library kernels only)
  C2C_STRIDED = 13, // rows with element strides and transform distances (k_c2c_strided, library kernels only)
};

// Four-step geometry of a length-N FFT beyond one CTA, N = n1 * n2.
struct FourStep {
  long long n;        // N
  int n1, n2;         // rows (column-FFT length) x row length
  int tw_shift;       // L = 2^tw_shift, L^2 >= N: the two-level inter-pass twiddle table
  const void* lo;     // w_N^e, e < L
  const void* hi;     // w_N^(e L), e < ceil(N / L)
  long long n_user;   // Bluestein: user length (inputs past it are zero, outputs dropped)
  const void* chirp;  // Bluestein: c_j, j < n_user
  const void* bhat;   // Bluestein: FFT_N(conj c) / N
};

// Pass A's per-CTA twiddle tables: tpb rows of ceil(n1 / 32) entries, then
// tpb rows of 32. The lanes of a warp read column t = lane % tpb, row
// offset j = lane / tpb: table A at one row offset for all lanes (an odd
// stride spreads the tpb rows over the banks), table B at t * S + j, which
// is conflict-free for S = 32 + 32 / tpb.
__host__ __device__ constexpr int smem_twiddle_stride_a(int n1) { return ((n1 + 31) / 32) | 1; }
__host__ __device__ constexpr int smem_twiddle_stride_b(int tpb) { return 32 + (tpb < 32 ? 32 / tpb : 1); }
__host__ __device__ constexpr int smem_twiddle_entries(int tpb, int n1) {
  return tpb * (smem_twiddle_stride_a(n1) + smem_twiddle_stride_b(tpb));
}

// GPU-scope acquire load of a dependency counter.
__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

#ifndef __CUDACC_RTC__
// Four-step passes: pass_a selects the column pass (mode 0 plain, 1 chirp
// input) or the transposing row pass (mode 0 plain, 1 spectrum, 2 chirp
// output, 3 the Bluestein middle pass k_rows_bb).
template <typename T>
cudaError_t launch_fourstep(bool pass_a, int mode, bool k1, const KArgs& a, const FourStep& fs, unsigned blocks,
                            unsigned threads, size_t smem, cudaStream_t stream);

// Launch `which` for dtype T (float or double) with `blocks` CTAs of
// `threads` threads and `smem` bytes of dynamic shared memory; `blue`
// selects the Bluestein core and `k1` the one-butterfly-per-thread variant.
template <typename T>
cudaError_t launch_kernel(Kernel which, bool blue, bool k1, const KArgs& a, unsigned blocks, unsigned threads,
                          size_t smem, cudaStream_t stream);
// Per-family launchers (k_complex_*.cu, k_real_*.cu), dispatched by launch_kernel.
template <typename T>
cudaError_t launch_complex(Kernel which, bool blue, bool k1, const KArgs& a, unsigned blocks, unsigned threads,
                           size_t smem, cudaStream_t stream);
template <typename T>
cudaError_t launch_real(Kernel which, bool blue, bool k1, const KArgs& a, unsigned blocks, unsigned threads,
                        size_t smem, cudaStream_t stream);

// Table generators (FP64 arithmetic, stored in the working dtype T).
enum class Table : int {
  OMEGA = 0,       // out[k] = exp(-2 pi i k / n), k < count
  CHIRP = 1,       // out[k] = exp(-pi i (k*k mod 2n) / n), k < count
  RCOEF = 2,       // out[k] = (1 + i omega_n^k) / 2
  RBCOEF = 3,      // out[k] = (1 - i omega_n^-k) / 2
  OMEGA4N_POS = 4, // out[k] = exp(+2 pi i k / (4n))
  OMEGA4N_NEG = 5, // out[k] = exp(-2 pi i k / (4n))
  MDCT_TW = 6,     // out[k] = exp(-2 pi i (8k+1) / (8n)) * (2/n)^(1/4)
  SINE_WIN = 7,    // real: sin(pi (k + 1/2) / n)
  VORBIS_WIN = 8,  // real: sin(pi/2 sin^2(pi (k + 1/2) / n))
  BLUE_B = 9,      // f64 only: Bluestein kernel sequence for user length n, padded length m, x 1/m
  CHIRP_INDEX = 10,// u64: k*k mod 2n
  OMEGA_STRIDE = 11 // out[k] = exp(-2 pi i (k*m mod n) / n)
};

template <typename T>
cudaError_t gen_table(Table which, long long n, long long count, long long m, void* out, cudaStream_t stream);

// Radices of a pass order (first pass first).
struct PassList {
  int npass;
  int r[24];
};
// Stage twiddle table of a pass order: for pass p (radix R, Ns = product of
// the earlier radices) the block [(R-1) x Ns] holds exp(-2 pi i jm r /
// (Ns R)) at (r-1)*Ns + jm; blocks follow pass order. prod(r) - 1 entries.
template <typename T>
cudaError_t gen_stage_table(const PassList& pl, void* out, cudaStream_t stream);

// Elementwise f64 -> T complex conversion (Bluestein spectrum rounding).
template <typename T>
cudaError_t convert_from_f64(const double2* src, void* dst, long long count, cudaStream_t stream);
#endif  // __CUDACC_RTC__

}  // namespace chfft
