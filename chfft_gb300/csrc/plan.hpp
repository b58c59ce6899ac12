// Host-side plan compiler: radix selection, Bluestein padding, table
// generation and launch geometry for the kernels in k_*.cu.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "kernels.cuh"

namespace chfft {

// Error carried from deep inside plan building / execution to the C ABI.
struct Fail {
  int code;
  std::string msg;
};

void cuda_check(cudaError_t e, const char* what);
#define CHFFT_CUDA(call) ::chfft::cuda_check((call), #call)

// Owning device allocation.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes) {
    o.p = nullptr;
    o.bytes = 0;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    release();
    p = o.p;
    bytes = o.bytes;
    o.p = nullptr;
    o.bytes = 0;
    return *this;
  }
  ~DevBuf() { release(); }
  void release();
  void ensure(size_t b);  // grow (contents not kept)
};

constexpr size_t kMaxSmem = 227 * 1024;  // dynamic shared memory per CTA on sm_103

inline int ept_of(int dtype) { return dtype == 0 ? 32 : 16; }
inline size_t cplx_bytes(int dtype) { return dtype == 0 ? 8 : 16; }
inline size_t real_bytes(int dtype) { return dtype == 0 ? 4 : 8; }

// 2^a 3^b 5^c 7^d, or ok = false.
struct Smooth {
  int e2 = 0, e3 = 0, e5 = 0, e7 = 0;
  bool ok = false;
};
Smooth factor_smooth(long long n);

// Stage list for a 7-smooth n (fewest passes; radices 16/8/4/2/10/5/3/7).
// Returns false when n is not 7-smooth.
bool make_stages(long long n, StageList* out);
// Threads a CTA needs to run `tpb` sequences with these stages (k1: one
// butterfly per thread per pass; otherwise up to EPT/R per thread).
int threads_needed(const StageList& st, int ept, int tpb, bool k1 = false);
// Whether one sequence of these stages fits a CTA (threads and shared memory).
bool fits_cta(const StageList& st, int dtype);
// Radices in the order the fused kernels run them (rf, mid..., rl), or the
// canonical order when the list has fewer than two passes.
std::vector<int> pass_order(const StageList& st);

// Complex core FFT of logical length n for one dtype: mixed radix when n is
// 7-smooth and fits a CTA, otherwise Bluestein with a 7-smooth M >= 2n-1.
struct Core {
  long long n = 0;
  int dtype = 0;
  bool blue = false;
  StageList st{};  // stages of the FFT actually run (length M for Bluestein)
  DevBuf tw, chirp, bhat, stw;
  bool build(long long n, int dtype, cudaStream_t s);  // false: unsupported size
  CoreDesc desc() const;
  long long fft_len() const { return st.n; }
  size_t device_bytes() const { return tw.bytes + chirp.bytes + bhat.bytes + stw.bytes; }
};

// Launch geometry of a CTA-per-`tpb`-sequences kernel.
struct Geo {
  int tpb = 1, threads = 32;
  size_t smem = 0;
  int ld = 0;
  bool k1 = false;  // one-butterfly-per-thread kernel variant
};
Geo row_geo(const Core& c, long long count, int target_threads = 256);
Geo col_geo(const Core& c, int ncols);

// Smallest 7-smooth M >= lo that the CTA engine runs cheapest (M * passes).
long long bluestein_length(long long n, int dtype);

// Whether plan-time specialised kernels are used for a launch of `elems`
// elements (CHFFT_JIT policy).
bool want_specialised(long long elems);

// Complex FFT of a length beyond one CTA: four-step N = n1 * n2 (column
// pass + transposing row pass, jit/library kernels), or Bluestein with a
// four-step M. The batch runs in chunks sized to keep the intermediate in L2.
struct BigCore {
  long long n = 0;  // logical length
  long long m = 0;  // FFT length run (n, or the Bluestein M)
  int dtype = 0;
  bool blue = false;
  int n1 = 0, n2 = 0, tw_l = 0;
  Core ca, cb;  // column core (n1), row core (n2)
  DevBuf lo, hi, chirp, bhat;
  bool build(long long n, int dtype, cudaStream_t s);  // false: unsupported
  FourStep fs() const;
  long long chunk(long long batch) const;                  // transforms per chunk
  long long work_elems(long long batch) const;             // complex workspace elements
  // batch contiguous sequences in -> out (distance n), workspace `work`.
  // max_chunk > 0 caps the transforms per chunk (a fixed-size workspace);
  // library_only skips plan-time specialised kernels.
  void exec(const void* in, void* out, void* work, long long batch, bool back, double scale, cudaStream_t s,
            long long max_chunk = 0, bool library_only = false) const;
  // Workspace bytes one transform needs.
  size_t work_bytes_per_transform() const { return (size_t)m * cplx_bytes(dtype) * (blue ? 2 : 1); }
  size_t device_bytes() const {
    return ca.device_bytes() + cb.device_bytes() + lo.bytes + hi.bytes + chirp.bytes + bhat.bytes;
  }
};

// Split of a 7-smooth m into n1 x n2 CTA-sized factors (false if none).
bool four_step_split(long long m, int dtype, int* n1, int* n2);

}  // namespace chfft
