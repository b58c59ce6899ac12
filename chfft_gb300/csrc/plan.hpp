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

// One page-locked int mapped into the device address space (cudaHostAlloc
// mapped): kernels write it, the host reads it after a synchronisation.
struct HostWord {
  int* host = nullptr;
  int* dev = nullptr;
  HostWord() = default;
  HostWord(const HostWord&) = delete;
  HostWord& operator=(const HostWord&) = delete;
  ~HostWord();
  void ensure();
  // The recorded code (0 if none), cleared.
  int take();
};

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

// Stage list for a 7-smooth n (fewest passes; radices 16/8/4/2/10/5/3/7,
// and 32 when max_radix is 32). Returns false when n is not 7-smooth.
bool make_stages(long long n, StageList* out, int max_radix = 16);
// Threads a CTA needs to run `tpb` sequences with these stages (k1: one
// butterfly per thread per pass; otherwise up to EPT/R per thread).
int threads_needed(const StageList& st, int ept, int tpb, bool k1 = false);
// Whether one sequence of these stages fits a CTA (threads and shared memory).
bool fits_cta(const StageList& st, int dtype);
// Radices in the order the fused kernels run them (rf, mid..., rl), or the
// canonical order when the list has fewer than two passes.
std::vector<int> pass_order(const StageList& st);

// Tuning knobs of a plan: the autotuner's search space. Zero or -1 leaves a
// knob to the built-in heuristic.
struct PlanOpts {
  int k1 = -1;           // one butterfly per thread (1), several (0), auto (-1)
  int tpb = 0;           // sequences per CTA (rows), 0 auto
  int max_radix = 0;     // specialised f32 kernels: 16 or 32 (0: 32)
  int jit = -1;          // specialised kernels: policy (-1), never (0), always (1)
  long long blue_m = 0;  // Bluestein length M (7-smooth, >= 2n - 1), 0 auto
  int fs_n1 = 0;         // four-step column length n1, 0 auto
  int fs_tpb = 0;        // four-step / 2-D column tile width, 0 auto
  int l2_mb = 0;         // four-step chunk budget in MiB, 0 auto (512)
  int tc = 0;            // f32 radix-16 passes on tensor cores: 0 off, 1 FP16x2, 2 BF16x2, 3 BF16x3
  int min_blocks = 0;    // specialised kernels: launch-bounds CTAs per SM, 0 auto
  int balance = -1;      // specialised kernels: balanced mixed-radix variant (-1 auto = on, 0 off, 1 on)
  int ept = 0;           // column kernels: elements per thread of the several-butterflies variant, 0 default
};

// Complex core FFT of logical length n for one dtype: mixed radix when n is
// 7-smooth and fits a CTA, otherwise Bluestein with a 7-smooth M >= 2n-1
// (blue_m when it is valid).
struct Core {
  long long n = 0;
  int dtype = 0;
  bool blue = false;
  StageList st{};  // stages of the FFT actually run (length M for Bluestein)
  // Radix-32 stage list for compile-time-stage kernels with 32 elements per
  // thread (f32), with its own stage twiddles; wide.p is null when it equals st.
  StageList sw{};
  // Tensor-core pass order (r0, 16, ..., 16), n = r0 * 16^tc_s16 (f32, power
  // of two), and its stage twiddles; tc_s16 = 0 when n does not qualify.
  int tc_r0 = 0, tc_s16 = 0;
  // Rader cores: a two-pass order (two radices of at most 64) for the
  // plan-time Rader kernels, and its stage twiddles; empty otherwise.
  std::vector<int> order2;
  DevBuf tw, chirp, bhat, stw, wide, tcw, stw2;
  bool build(long long n, int dtype, cudaStream_t s, long long blue_m = 0);  // false: unsupported size
  void build_wide(cudaStream_t s);  // also the tensor-core pass order
  void build_tc(cudaStream_t s);
  CoreDesc desc() const;
  long long fft_len() const { return st.n; }
  size_t device_bytes() const {
    return tw.bytes + chirp.bytes + bhat.bytes + stw.bytes + wide.bytes + tcw.bytes + stw2.bytes;
  }
};

// Rader's algorithm for a prime n whose n - 1 = L is 7-smooth and fits one
// CTA (k_c2c_rader): the L-point core, the permutations g^p and g^-q mod n
// (g the least primitive root), and B^ = FFT_L(b) / L, b_m = w_n^(g^-m),
// computed in FP64 and rounded once.
struct RaderCore {
  long long n = 0;
  int L = 0, g = 0, dtype = 0;
  Core lc;
  DevBuf perm, bhat;
  bool build(long long n, int dtype, cudaStream_t s);  // false: n does not qualify
  void release() {
    n = 0;
    perm.release();
    bhat.release();
  }
  size_t device_bytes() const { return lc.device_bytes() + perm.bytes + bhat.bytes; }
};

// Latency form of small CFft1D batches (k_cluster.cuh): one transform per
// thread-block cluster of csize CTAs, N = n1 x n2 split over the cluster
// (each CTA n2 / csize columns, then n1 / csize rows), the exchange through
// distributed shared memory. Built for 7-smooth lengths with such a split;
// used for batches of at most max_batch transforms.
struct ClusterCore {
  long long n = 0;
  int dtype = 0, n1 = 0, n2 = 0, csize = 0, threads = 0, lda = 0, ldb = 0, tsz = 0;
  int npa = 0, npb = 0;
  unsigned long long code_a = 0, code_b = 0;  // radix of pass p at bits [4p, 4p + 4)
  size_t smem = 0;
  long long max_batch = 0;
  const void* fn = nullptr;  // the kernel (compile-time-shape instance or the run-time-shape one)
  DevBuf tab_a, tab_b;  // per-pass input twiddles of the n1- and n2-point FFTs
  // Four-step twiddles x scale ([n2][k1]) for the scales of the CFft1D
  // methods: 1, 1 / sqrt(n), 1 / n.
  static constexpr int kScales = 3;
  double scales[kScales] = {};
  DevBuf blk[kScales];
  // Host-mapped error word: 7 when a CTA's wait for its rows gave up.
  HostWord err;
  // false: no split, no cluster shape that launches, CHFFT_CLUSTER=0, or
  // (beyond_cta: the plan's own path is the four-step one) a length where
  // the four-step launches are faster.
  bool build(long long n, int dtype, cudaStream_t s, bool beyond_cta = false);
  void release() {
    n = 0;
    max_batch = 0;
    tab_a.release();
    tab_b.release();
    for (auto& b : blk) b.release();
  }
  // false (nothing launched) for a scale without a table.
  bool exec(const void* in, void* out, long long batch, bool back, double scale, cudaStream_t s) const;
  size_t device_bytes() const {
    size_t b = tab_a.bytes + tab_b.bytes;
    for (const auto& x : blk) b += x.bytes;
    return b;
  }
};

// Launch geometry of a CTA-per-`tpb`-sequences kernel.
struct Geo {
  int tpb = 1, threads = 32;
  size_t smem = 0;
  int ld = 0;
  bool k1 = false;     // one-butterfly-per-thread kernel variant
  int max_radix = 32;  // compile-time-stage kernels: 32 allows the core's radix-32 list
  int min_blocks = 0;  // compile-time-stage kernels: launch-bounds CTAs per SM (0: 2 for k1, else 1)
  int ept = 0;         // compile-time-stage kernels: elements per thread of the several-butterflies variant
  int balance = -1;    // compile-time-stage kernels: balanced variant of a mixed-radix k1 geometry (-1 auto, 0 off)
};
Geo row_geo(const Core& c, long long count, const PlanOpts& o = PlanOpts{});
Geo col_geo(const Core& c, int ncols, int tpb_opt = 0, const PlanOpts& o = PlanOpts{});
// Rader rows: the L-point core's geometry with the staged rows (stride
// *ldr) and X_0 slots added to the shared memory.
Geo rader_geo(const RaderCore& r, long long count, const PlanOpts& o, int* ldr);

// Smallest 7-smooth M >= lo that the CTA engine runs cheapest (M * passes).
long long bluestein_length(long long n, int dtype);

// Polls a bounded device-side wait makes before it gives up: CHFFT_SPIN_LIMIT,
// default 4,000,000 (about a second at ~0.25 us per poll).
long long spin_limit();
// Test hook: CHFFT_TEST_STALL=1 makes one dependency of each pipelined
// four-step launch, and the rows' arrival wait of each cluster launch,
// unreachable, so a bounded wait runs out and the call reports
// CHFFT_ETIMEOUT (the kernels still return normally).
int stall_test();

// Whether plan-time specialised kernels are used for a launch of `elems`
// elements (CHFFT_JIT policy, unless the plan's jit knob overrides it).
bool want_specialised(long long elems, int jit_opt = -1);

// Complex FFT of a length beyond one CTA: four-step N = n1 * n2 (column
// pass + transposing row pass, jit/library kernels), or Bluestein with a
// four-step M. The batch runs in chunks sized to keep the intermediate in L2.
struct BigCore {
  long long n = 0;  // logical length
  long long m = 0;  // FFT length run (n, or the Bluestein M)
  int dtype = 0;
  bool blue = false;
  int n1 = 0, n2 = 0, tw_l = 0, tw_shift = 0;
  Core ca, cb;  // column core (n1), row core (n2)
  DevBuf lo, hi, chirp, bhat;
  // Pipelined four-step (k_pipe.cuh): both passes in one persistent launch,
  // for f32 non-Bluestein lengths whose split has a kernel shape. Stage
  // twiddles of the (n/32, 32) pass orders of n1 and n2, and the pass-A
  // tiles' twiddle tables.
  bool pipe = false;
  DevBuf pstw_a, pstw_b, ptw;
  // Host-mapped error word the pipelined launch sets when a bounded wait
  // gives up; read (and cleared) after the plan's stream is synchronised.
  HostWord err;
  PlanOpts opts;
  bool build(long long n, int dtype, cudaStream_t s, const PlanOpts& o = PlanOpts{});  // false: unsupported
  FourStep fs() const;
  long long chunk(long long batch) const;                  // transforms per chunk
  long long work_elems(long long batch) const;             // complex workspace elements
  // Pipelined launch parameters for `batch` transforms (ring slots, lead,
  // L2 hints); false when the pipelined kernel does not apply.
  bool pipe_params(long long batch, int* ring, int* lead, int* hints) const;
  // batch contiguous sequences in -> out (distance n), workspace `work`.
  // max_chunk > 0 caps the transforms per chunk (a fixed-size workspace);
  // library_only skips plan-time specialised kernels.
  void exec(const void* in, void* out, void* work, long long batch, bool back, double scale, cudaStream_t s,
            long long max_chunk = 0, bool library_only = false) const;
  // Workspace bytes one transform needs.
  size_t work_bytes_per_transform() const { return (size_t)m * cplx_bytes(dtype) * (blue ? 2 : 1); }
  size_t device_bytes() const {
    return ca.device_bytes() + cb.device_bytes() + lo.bytes + hi.bytes + chirp.bytes + bhat.bytes + pstw_a.bytes +
           pstw_b.bytes + ptw.bytes;
  }
};

// Split of a 7-smooth m into n1 x n2 CTA-sized factors (false if none).
bool four_step_split(long long m, int dtype, int* n1, int* n2);
// Smallest s with (2^s)^2 >= m: the inter-pass twiddle split w^e = hi[e >> s] lo[e & (2^s - 1)].
inline int tw_shift_for(long long m) {
  int s = 0;
  while ((1LL << (2 * s)) < m) s++;
  return s;
}

}  // namespace chfft
