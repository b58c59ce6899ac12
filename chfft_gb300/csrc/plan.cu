// Plan compiler: radix selection, Bluestein padding and the FP64-generated
// tables of a complex core FFT, plus launch geometry.
//
// chfft picks mixed radix when N is 7-smooth and Chirp-Z otherwise, with
// M = next_pow2(N) << 1 (src/cfft1d.rs:103-206). The same split is kept;
// the radices differ (16/8/4/2/10/5/3/7 Stockham passes instead of chfft's
// 4/2/3/5/generic DIT stages, src/mixed_radix.rs:104-166) and M is the
// cheapest 7-smooth length >= 2N-1, which gives the same convolution.
#include "plan.hpp"

#include <algorithm>
#include <utility>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "../../include/chfft_gpu.h"
#include "jit.hpp"
#include "cluster.hpp"
#include "k_cluster.cuh"
#include "k_pipe.cuh"
#include "pipe.hpp"

namespace chfft {

void cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  int code = (e == cudaErrorMemoryAllocation) ? 5 /*CHFFT_ENOMEM*/ : 4 /*CHFFT_ECUDA*/;
  throw Fail{code, std::string(what) + ": " + cudaGetErrorString(e)};
}

HostWord::~HostWord() {
  if (host) cudaFreeHost(host);
}

void HostWord::ensure() {
  if (host) return;
  void* h = nullptr;
  CHFFT_CUDA(cudaHostAlloc(&h, sizeof(int), cudaHostAllocMapped));
  host = static_cast<int*>(h);
  *host = 0;
  void* d = nullptr;
  cudaError_t e = cudaHostGetDevicePointer(&d, h, 0);
  if (e != cudaSuccess) {
    cudaFreeHost(h);
    host = nullptr;
    cuda_check(e, "cudaHostGetDevicePointer");
  }
  dev = static_cast<int*>(d);
}

int HostWord::take() {
  if (!host) return 0;
  const int v = *(volatile int*)host;
  if (v) *(volatile int*)host = 0;
  return v;
}

void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

void DevBuf::ensure(size_t b) {
  if (b <= bytes && p) return;
  release();
  if (b == 0) return;
  CHFFT_CUDA(cudaMalloc(&p, b));
  bytes = b;
}

Smooth factor_smooth(long long n) {
  Smooth s;
  if (n <= 0) return s;
  while (n % 2 == 0) n /= 2, s.e2++;
  while (n % 3 == 0) n /= 3, s.e3++;
  while (n % 5 == 0) n /= 5, s.e5++;
  while (n % 7 == 0) n /= 7, s.e7++;
  s.ok = (n == 1);
  return s;
}

static int radix_index(int r) {
  for (int i = 0; i < kNumRadix; i++)
    if (radix_at(i) == r) return i;
  return -1;
}

bool make_stages(long long n, StageList* out, int max_radix) {
  StageList st{};
  st.n = (int)n;
  Smooth s = factor_smooth(n);
  if (!s.ok || n > INT_MAX) return false;
  const int maxbits = max_radix >= 32 ? 5 : 4;
  // t radix-10 passes absorb t twos and t fives; choose t for fewest passes.
  int best_t = 0, best_passes = INT_MAX;
  for (int t = 0; t <= std::min(s.e2, s.e5); t++) {
    int twos = s.e2 - t;
    int passes = s.e7 + s.e3 + (s.e5 - t) + t + (twos + maxbits - 1) / maxbits;
    if (passes < best_passes || (passes == best_passes && t > best_t)) {
      best_passes = passes;
      best_t = t;
    }
  }
  int cnt[kNumRadix] = {0};
  cnt[radix_index(10)] = best_t;
  cnt[radix_index(5)] = s.e5 - best_t;
  cnt[radix_index(3)] = s.e3;
  cnt[radix_index(7)] = s.e7;
  // Powers of two: p = ceil(twos/maxbits) passes of near-equal size.
  int twos = s.e2 - best_t;
  int p2 = (twos + maxbits - 1) / maxbits;
  for (int i = 0; i < p2; i++) {
    int bits = twos / p2 + (i < twos % p2 ? 1 : 0);
    cnt[radix_index(1 << bits)]++;
  }
  st.npass = 0;
  for (int i = 0; i < kNumRadix; i++) {
    st.all[i] = cnt[i];
    st.mid[i] = cnt[i];
    st.npass += cnt[i];
  }
  st.rf = st.rl = 0;
  if (st.npass >= 2) {
    for (int i = 0; i < kNumRadix; i++)
      if (st.mid[i] > 0) {
        st.rf = radix_at(i);
        st.mid[i]--;
        break;
      }
    for (int i = kNumRadix - 1; i >= 0; i--)
      if (st.mid[i] > 0) {
        st.rl = radix_at(i);
        st.mid[i]--;
        break;
      }
  }
  *out = st;
  return true;
}

int threads_needed(const StageList& st, int ept, int tpb, bool k1) {
  long long need = 1;
  for (int i = 0; i < kNumRadix; i++) {
    if (st.all[i] == 0) continue;
    int r = radix_at(i);
    long long k = k1 ? 1 : ept / r;
    long long nb = (long long)tpb * (st.n / r);
    need = std::max(need, (nb + k - 1) / k);
  }
  return (int)std::min<long long>(need, INT_MAX);
}

std::vector<int> pass_order(const StageList& st) {
  std::vector<int> r;
  if (st.npass >= 2) {
    r.push_back(st.rf);
    for (int i = 0; i < kNumRadix; i++)
      for (int c = 0; c < st.mid[i]; c++) r.push_back(radix_at(i));
    r.push_back(st.rl);
  } else {
    for (int i = 0; i < kNumRadix; i++)
      for (int c = 0; c < st.all[i]; c++) r.push_back(radix_at(i));
  }
  return r;
}

// Stage twiddles for the fused pass order (compile-time-stage kernels).
static void build_stage_table(DevBuf& buf, const StageList& st, int dtype, cudaStream_t s) {
  std::vector<int> order = pass_order(st);
  PassList pl{};
  pl.npass = (int)order.size();
  for (size_t i = 0; i < order.size(); i++) pl.r[i] = order[i];
  buf.ensure((size_t)std::max(st.n - 1, 1) * cplx_bytes(dtype));
  CHFFT_CUDA(dtype == 0 ? gen_stage_table<float>(pl, buf.p, s) : gen_stage_table<double>(pl, buf.p, s));
}

bool fits_cta(const StageList& st, int dtype) {
  if (threads_needed(st, ept_of(dtype), 1) > kMaxThreads) return false;
  return (size_t)smem_ld(st.n) * cplx_bytes(dtype) <= kMaxSmem;
}

long long bluestein_length(long long n, int dtype) {
  long long lo = 2 * n - 1, best = -1;
  double best_cost = 1e300;
  long long hi = 1;
  while (hi < lo) hi <<= 1;
  for (long long m = lo; m <= hi; m++) {
    StageList st;
    if (!make_stages(m, &st) || !fits_cta(st, dtype)) continue;
    double cost = (double)m * (st.npass + 0.5);
    if (cost < best_cost) {
      best_cost = cost;
      best = m;
    }
  }
  return best;
}

static void fft_f64_inplace(double2* d_data, const Core& c64, cudaStream_t s);

void Core::build_tc(cudaStream_t s) {
  tc_r0 = tc_s16 = 0;
  tcw.release();
  const int m = st.n;
  if (dtype != 0 || m < 16 || (m & (m - 1))) return;
  int k = 0;
  while ((1 << k) < m) k++;
  PassList pl{};
  const int r0 = 1 << (k % 4);
  if (r0 > 1) pl.r[pl.npass++] = r0;
  for (int i = 0; i < k / 4; i++) pl.r[pl.npass++] = 16;
  tcw.ensure((size_t)std::max(m - 1, 1) * cplx_bytes(dtype));
  CHFFT_CUDA(gen_stage_table<float>(pl, tcw.p, s));
  tc_r0 = r0;
  tc_s16 = k / 4;
}

void Core::build_wide(cudaStream_t s) {
  build_tc(s);
  sw = st;
  wide.release();
  if (dtype != 0 || st.n < 2) return;
  StageList w;
  if (!make_stages(st.n, &w, 32) || pass_order(w) == pass_order(st)) return;
  sw = w;
  build_stage_table(wide, sw, dtype, s);
}

bool Core::build(long long n_, int dtype_, cudaStream_t s, long long blue_m) {
  n = n_;
  dtype = dtype_;
  blue = false;
  tw.release();
  chirp.release();
  bhat.release();
  stw.release();
  wide.release();
  tcw.release();
  order2.clear();
  stw2.release();
  tc_r0 = tc_s16 = 0;
  const size_t cb = cplx_bytes(dtype);
  if (n == 1) {
    st = StageList{};
    st.n = 1;
    sw = st;
    return true;
  }
  if (make_stages(n, &st) && fits_cta(st, dtype)) {
    tw.ensure(n * cb);
    CHFFT_CUDA(dtype == 0 ? gen_table<float>(Table::OMEGA, n, n, 0, tw.p, s)
                          : gen_table<double>(Table::OMEGA, n, n, 0, tw.p, s));
    build_stage_table(stw, st, dtype, s);
    build_wide(s);
    return true;
  }
  // Bluestein core (src/chirpz.rs): chirp table and the spectrum of the
  // conjugate chirp, both from FP64.
  long long m = bluestein_length(n, dtype);
  if (m < 0) return false;
  StageList sb;
  if (blue_m >= 2 * n - 1 && make_stages(blue_m, &sb) && fits_cta(sb, dtype)) m = blue_m;
  blue = true;
  make_stages(m, &st);
  tw.ensure(m * cb);
  chirp.ensure(n * cb);
  bhat.ensure(m * cb);
  CHFFT_CUDA(dtype == 0 ? gen_table<float>(Table::OMEGA, m, m, 0, tw.p, s)
                        : gen_table<double>(Table::OMEGA, m, m, 0, tw.p, s));
  CHFFT_CUDA(dtype == 0 ? gen_table<float>(Table::CHIRP, n, n, 0, chirp.p, s)
                        : gen_table<double>(Table::CHIRP, n, n, 0, chirp.p, s));
  build_stage_table(stw, st, dtype, s);
  build_wide(s);
  // B^ = FFT_M(b) / M in FP64 when the f64 engine can run length M in one
  // CTA; otherwise the FFT of the FP64 sequence runs in the working dtype.
  DevBuf b64;
  b64.ensure(m * sizeof(double2));
  CHFFT_CUDA(gen_table<double>(Table::BLUE_B, n, m, m, b64.p, s));
  Core c64;
  StageList st64;
  if (make_stages(m, &st64) && fits_cta(st64, 1)) {
    c64.build(m, 1, s);
    fft_f64_inplace(static_cast<double2*>(b64.p), c64, s);
    if (dtype == 0)
      CHFFT_CUDA(convert_from_f64<float>(static_cast<const double2*>(b64.p), bhat.p, m, s));
    else
      CHFFT_CUDA(cudaMemcpyAsync(bhat.p, b64.p, m * sizeof(double2), cudaMemcpyDeviceToDevice, s));
  } else {
    CHFFT_CUDA(convert_from_f64<float>(static_cast<const double2*>(b64.p), bhat.p, m, s));
    Core cm;
    cm.build(m, 0, s);
    KArgs a{};
    a.core = cm.desc();
    Geo g = row_geo(cm, 1);
    a.tpb = g.tpb;
    a.ld = g.ld;
    a.count = 1;
    a.in = bhat.p;
    a.out = bhat.p;
    a.scale = 1.0;
    a.in_dist = a.out_dist = m;
    CHFFT_CUDA(launch_kernel<float>(Kernel::C2C, false, g.k1, a, 1, g.threads, g.smem, s));
  }
  CHFFT_CUDA(cudaStreamSynchronize(s));  // temporaries are freed on return
  return true;
}

CoreDesc Core::desc() const {
  CoreDesc d{};
  d.st = st;
  d.tw = tw.p;
  d.n = (int)n;
  d.chirp = chirp.p;
  d.bhat = bhat.p;
  d.stw = stw.p;
  return d;
}

static void fft_f64_inplace(double2* d_data, const Core& c64, cudaStream_t s) {
  KArgs a{};
  a.core = c64.desc();
  Geo g = row_geo(c64, 1);
  a.tpb = g.tpb;
  a.ld = g.ld;
  a.count = 1;
  a.in = d_data;
  a.out = d_data;
  a.scale = 1.0;
  a.in_dist = a.out_dist = c64.st.n;
  CHFFT_CUDA(launch_kernel<double>(Kernel::C2C, false, g.k1, a, 1, g.threads, g.smem, s));
}

Geo row_geo(const Core& c, long long count, const PlanOpts& o) {
  Geo g;
  g.max_radix = o.max_radix == 16 ? 16 : 32;
  g.min_blocks = o.min_blocks;
  g.balance = o.balance;
  const int ept = ept_of(c.dtype);
  const int m = c.st.n;
  g.ld = smem_ld(m);
  const size_t per = (size_t)g.ld * cplx_bytes(c.dtype);
  const int t1k = std::max(1, threads_needed(c.st, ept, 1, true));
  const bool k1 = t1k <= kMaxThreads && o.k1 != 0;
  if (k1) {
    // One butterfly per thread: sequences up to about 256 threads per CTA
    // (the autotuner's pick on GB300: N=1000 2 sequences, 26.6 -> 19.8 us;
    // N=4096 1 sequence, 213 -> 189 us for 16384), keeping two CTAs' tiles
    // within an SM's shared memory.
    g.k1 = true;
    int tpb = o.tpb > 0 ? std::min(o.tpb, kMaxThreads / t1k) : std::max(1, 256 / t1k);
    tpb = (int)std::min<size_t>(tpb, std::max<size_t>(1, (o.tpb > 0 ? kMaxSmem : kMaxSmem / 2) / per));
    tpb = (int)std::max<long long>(1, std::min<long long>(tpb, count));
    g.tpb = tpb;
  } else {
    const int t1 = std::max(1, threads_needed(c.st, ept, 1));
    int tpb = o.tpb > 0 ? o.tpb : std::max(1, 256 / t1);
    tpb = (int)std::min<size_t>(tpb, std::max<size_t>(1, (o.tpb > 0 ? kMaxSmem : 64 * 1024) / per));
    tpb = (int)std::max<long long>(1, std::min<long long>(tpb, count));
    while (tpb > 1 && threads_needed(c.st, ept, tpb) > kMaxThreads) tpb--;
    g.tpb = tpb;
  }
  int th = threads_needed(c.st, ept, g.tpb, g.k1);
  th = std::max(32, ((th + 31) / 32) * 32);
  g.threads = std::min(th, kMaxThreads);
  g.smem = (size_t)g.tpb * per;
  return g;
}

Geo rader_geo(const RaderCore& r, long long count, const PlanOpts& o, int* ldr) {
  // Several butterflies per thread unless the k1 knob asks otherwise: the
  // (n - 1)-point cores mix radices 16, 7 and 3 (1008 = 16 3 3 7), whose
  // one-butterfly geometry leaves most threads idle in the radix-16 pass.
  PlanOpts q = o;
  if (q.k1 < 0) q.k1 = 0;
  Geo g = row_geo(r.lc, count, q);
  *ldr = (int)(r.n | 1);
  const size_t cb = cplx_bytes(r.dtype);
  auto smem_for = [&](int tpb) {
    return ((size_t)tpb * g.ld * cb + 15) / 16 * 16 + (size_t)tpb * (*ldr + 1) * cb;
  };
  // Keep two CTAs' tiles within an SM's shared memory, as row_geo does.
  while (g.tpb > 1 && smem_for(g.tpb) > kMaxSmem / 2) g.tpb--;
  g.threads = std::min(kMaxThreads, std::max(32, (threads_needed(r.lc.st, ept_of(r.dtype), g.tpb, g.k1) + 31) / 32 * 32));
  g.smem = smem_for(g.tpb);
  return g;
}

namespace {
long long mulmod(long long a, long long b, long long m) { return (long long)((__int128)a * b % m); }
long long powmod(long long a, long long e, long long m) {
  long long r = 1 % m;
  a %= m;
  for (; e > 0; e >>= 1, a = mulmod(a, a, m))
    if (e & 1) r = mulmod(r, a, m);
  return r;
}
bool is_prime(long long n) {
  if (n < 2) return false;
  for (long long d = 2; d * d <= n; d++)
    if (n % d == 0) return false;
  return true;
}
}  // namespace

bool RaderCore::build(long long n_, int dtype_, cudaStream_t s) {
  release();
  const long long L_ = n_ - 1;
  if (n_ < 11 || n_ > (1LL << 24) || !is_prime(n_)) return false;
  StageList st;
  if (!make_stages(L_, &st) || !fits_cta(st, dtype_)) return false;
  // One sequence's tile, staged row and X_0 slot must fit a CTA (with room
  // for the plan-time kernels' wider tile stride).
  const size_t cb = cplx_bytes(dtype_);
  if ((size_t)(smem_ld(L_) + 64) * cb + (size_t)((n_ | 1) + 1) * cb + 16 > kMaxSmem) return false;
  // The least primitive root: g^(L/q) != 1 for every prime q | L (q in 2, 3, 5, 7).
  int root = 0;
  for (int cand = 2; cand < n_ && !root; cand++) {
    bool ok = true;
    for (int q : {2, 3, 5, 7})
      if (L_ % q == 0 && powmod(cand, L_ / q, n_) == 1) ok = false;
    if (ok) root = cand;
  }
  if (!root || !lc.build(L_, dtype_, s)) return false;
  // Two passes for the plan-time f32 kernels: L = r1 r2 with both radices at
  // most 64, as close to sqrt(L) as possible (1008 = 28 x 36). (f64 keeps the
  // standard order: 64 complex doubles per thread spill.)
  lc.order2.clear();
  lc.stw2.release();
  for (long long d = 2, best = 1LL << 40; dtype_ == 0 && d <= 64; d++) {
    if (L_ % d || L_ / d > 64 || !factor_smooth(d).ok || !factor_smooth(L_ / d).ok) continue;
    const long long spread = std::llabs(L_ / d - d);
    if (spread < best || (spread == best && d < L_ / d)) {
      best = spread;
      lc.order2 = {(int)d, (int)(L_ / d)};
    }
  }
  if (!lc.order2.empty()) {
    PassList pl{};
    pl.npass = 2;
    pl.r[0] = lc.order2[0];
    pl.r[1] = lc.order2[1];
    lc.stw2.ensure((size_t)(L_ - 1) * cplx_bytes(dtype_));
    CHFFT_CUDA(dtype_ == 0 ? gen_stage_table<float>(pl, lc.stw2.p, s) : gen_stage_table<double>(pl, lc.stw2.p, s));
  }
  n = n_;
  L = (int)L_;
  g = root;
  dtype = dtype_;
  std::vector<int> pm(2 * (size_t)L);
  std::vector<double2> b(L);
  const long long ginv = powmod(root, L_ - 1, n_);
  long long gp = 1, gq = 1;
  for (int i = 0; i < L; i++) {
    pm[i] = (int)gp;        // g^i
    pm[L + i] = (int)gq;    // g^-i
    // b_i = w_n^(g^-i) / L, FP64 with the numerator reduced to (-n/2, n/2]
    long long e = gq;
    if (2 * e > n_) e -= n_;
    const double ang = -2.0 * M_PI * (double)e / (double)n_;
    b[i] = make_double2(std::cos(ang) / (double)L, std::sin(ang) / (double)L);
    gp = mulmod(gp, root, n_);
    gq = mulmod(gq, ginv, n_);
  }
  perm.ensure(pm.size() * sizeof(int));
  CHFFT_CUDA(cudaMemcpyAsync(perm.p, pm.data(), pm.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  // B^ = FFT_L(b) by the FP64 core, rounded once to the working dtype.
  DevBuf b64;
  b64.ensure((size_t)L * sizeof(double2));
  CHFFT_CUDA(cudaMemcpyAsync(b64.p, b.data(), (size_t)L * sizeof(double2), cudaMemcpyHostToDevice, s));
  StageList st64;
  if (make_stages(L_, &st64) && fits_cta(st64, 1)) {
    Core c64;
    if (!c64.build(L_, 1, s)) return false;
    fft_f64_inplace(static_cast<double2*>(b64.p), c64, s);
  } else {  // the FP64 four-step engine
    BigCore big64;
    DevBuf w64;
    if (!big64.build(L_, 1, s)) return false;
    w64.ensure(big64.work_elems(1) * sizeof(double2));
    big64.exec(b64.p, b64.p, w64.p, 1, false, 1.0, s);
    CHFFT_CUDA(cudaStreamSynchronize(s));
  }
  bhat.ensure((size_t)L * cplx_bytes(dtype));
  if (dtype == 0)
    CHFFT_CUDA(convert_from_f64<float>(static_cast<const double2*>(b64.p), bhat.p, L, s));
  else
    CHFFT_CUDA(cudaMemcpyAsync(bhat.p, b64.p, (size_t)L * sizeof(double2), cudaMemcpyDeviceToDevice, s));
  CHFFT_CUDA(cudaStreamSynchronize(s));  // the host tables and b64 are freed on return
  return true;
}

Geo col_geo(const Core& c, int ncols, int tpb_opt, const PlanOpts& o) {
  Geo g;
  g.max_radix = o.max_radix == 16 ? 16 : 32;
  g.min_blocks = o.min_blocks;
  g.balance = o.balance;
  // Elements per thread of the several-butterflies variant: the dtype's
  // default, or the `ept` knob (specialised kernels; a library kernel keeps
  // its own and leaves the extra threads idle).
  const int ept = o.ept > 0 ? o.ept : ept_of(c.dtype);
  g.ld = smem_ld(c.st.n);
  const size_t per = (size_t)g.ld * cplx_bytes(c.dtype);
  int tpb = tpb_opt > 0 ? tpb_opt : (c.dtype == 0 ? 16 : 8);  // 128-byte row segments
  tpb = std::min(tpb, std::max(1, ncols));
  while (tpb > 1 && ((size_t)tpb * per > kMaxSmem || threads_needed(c.st, ept, tpb) > kMaxThreads)) tpb--;
  g.tpb = tpb;
  g.k1 = o.k1 != 0 && threads_needed(c.st, ept, tpb, true) <= kMaxThreads;
  if (!g.k1 && o.ept > 0) g.ept = o.ept;
  int th = threads_needed(c.st, ept, tpb, g.k1);
  th = std::max(32, ((th + 31) / 32) * 32);
  g.threads = std::min(th, kMaxThreads);
  g.smem = (size_t)tpb * per;
  return g;
}

long long spin_limit() {
  if (const char* e = std::getenv("CHFFT_SPIN_LIMIT")) {
    const long long v = std::atoll(e);
    if (v > 0) return v;
  }
  return 4000000;
}

int stall_test() {
  const char* e = std::getenv("CHFFT_TEST_STALL");
  return (e && e[0] == '1') ? 1 : 0;
}

bool want_specialised(long long elems, int jit_opt) {
  if (jit_opt >= 0) return jit_opt == 1;
  const JitMode mode = jit_mode();
  return mode == JitMode::ALWAYS || (mode == JitMode::AUTO && elems >= (1LL << 18));
}

// ---------------------------------------------------------------- four-step
bool four_step_split(long long m, int dtype, int* n1, int* n2) {
  const long long col_cap = dtype == 0 ? 2048 : 1024;  // column tiles of >= 8 columns
  double best = 1e300;
  bool ok = false;
  for (long long d = 2; d <= col_cap && d * d <= 4 * m; d++) {
    if (m % d) continue;
    const long long e = m / d;
    StageList s1, s2;
    if (!make_stages(d, &s1) || !make_stages(e, &s2) || !fits_cta(s1, dtype) || !fits_cta(s2, dtype)) continue;
    const double score = std::fabs(std::log((double)d) - 0.5 * std::log((double)m)) + (d > e ? 0.01 : 0.0);
    if (score < best) {
      best = score;
      *n1 = (int)d;
      *n2 = (int)e;
      ok = true;
    }
  }
  return ok;
}

static void launch_pass(bool pass_a, int mode, const Core& c, const Geo& g, const KArgs& a, const FourStep& fs,
                        unsigned blocks, long long elems, cudaStream_t s, bool library_only, int jit_opt, int tc) {
  // Plan-time pass-A kernels build their twiddle tables in shared memory (mode bit 3).
  const int jmode = mode | (pass_a && tc <= 0 ? 8 : 0);
  if (tc > 0 && !library_only) {
    const int r = jit_launch_tc(pass_a ? Kernel::COLS_TW : Kernel::ROWS_T, c, tc, g.tpb, a, blocks, s, jmode, &fs);
    if (r == 2) throw Fail{CHFFT_ECUDA, "launch of a tensor-core kernel failed"};
    if (r == 1) throw Fail{CHFFT_EUNSUPPORTED, "tensor-core kernel unavailable (plan compiler or geometry)"};
    return;
  }
  const Kernel kk = pass_a ? Kernel::COLS_TW : (mode == 3 ? Kernel::ROWS_BB : Kernel::ROWS_T);
  if (!library_only && want_specialised(elems, jit_opt) && jit_launch(kk, c.dtype, c, g, a, blocks, s, jmode, &fs) == 0)
    return;
  CHFFT_CUDA(c.dtype == 0 ? launch_fourstep<float>(pass_a, mode, g.k1, a, fs, blocks, g.threads, g.smem, s)
                          : launch_fourstep<double>(pass_a, mode, g.k1, a, fs, blocks, g.threads, g.smem, s));
}

bool BigCore::build(long long n_, int dtype_, cudaStream_t s, const PlanOpts& o) {
  n = n_;
  dtype = dtype_;
  blue = false;
  m = n;
  opts = o;
  const size_t cb_ = cplx_bytes(dtype);
  auto split = [&](long long len, int* a1, int* a2) {
    if (o.fs_n1 > 1 && len % o.fs_n1 == 0) {
      StageList s1, s2;
      const long long e = len / o.fs_n1;
      if (make_stages(o.fs_n1, &s1) && make_stages(e, &s2) && fits_cta(s1, dtype) && fits_cta(s2, dtype)) {
        *a1 = o.fs_n1;
        *a2 = (int)e;
        return true;
      }
    }
    return four_step_split(len, dtype, a1, a2);
  };
  if (!split(n, &n1, &n2)) {
    // Bluestein with a four-step M >= 2n - 1 (cheapest by M * passes).
    long long lo_m = 2 * n - 1, hi_m = 1, best_m = -1;
    while (hi_m < lo_m) hi_m <<= 1;
    double best = 1e300;
    for (long long mm = lo_m; mm <= hi_m; mm++) {
      int a1, a2;
      if (!factor_smooth(mm).ok || !four_step_split(mm, dtype, &a1, &a2)) continue;
      StageList s1, s2;
      make_stages(a1, &s1);
      make_stages(a2, &s2);
      const double cost = (double)mm * (s1.npass + s2.npass + 1);
      if (cost < best) {
        best = cost;
        best_m = mm;
      }
    }
    if (best_m < 0) return false;
    if (o.blue_m >= lo_m && factor_smooth(o.blue_m).ok && four_step_split(o.blue_m, dtype, &n1, &n2)) best_m = o.blue_m;
    blue = true;
    m = best_m;
    split(m, &n1, &n2);
  }
  if (!ca.build(n1, dtype, s) || !cb.build(n2, dtype, s)) return false;
  pipe = false;
  pstw_a.release();
  pstw_b.release();
  ptw.release();
  if (!blue && dtype == 0 && pipe_shape_ok(n1, n2)) {
    // Stage twiddles of the pipelined kernel's pass order (n/32, 32).
    for (int side = 0; side < 2; side++) {
      const int len = side ? n2 : n1;
      PassList pl{};
      pl.npass = 2;
      pl.r[0] = len / 32;
      pl.r[1] = 32;
      DevBuf& b = side ? pstw_b : pstw_a;
      b.ensure((size_t)(len - 1) * cb_);
      CHFFT_CUDA(gen_stage_table<float>(pl, b.p, s));
    }
    ptw.ensure(pipe_twiddle_elems(n1, n2) * cb_);
    CHFFT_CUDA(pipe_twiddles(n1, n2, ptw.p, s));
    err.ensure();
    pipe = true;
  }
  tw_shift = tw_shift_for(m);
  tw_l = 1 << tw_shift;
  const long long nhi = (m + tw_l - 1) / tw_l;
  lo.ensure(tw_l * cb_);
  hi.ensure(nhi * cb_);
  CHFFT_CUDA(dtype == 0 ? gen_table<float>(Table::OMEGA, m, tw_l, 0, lo.p, s)
                        : gen_table<double>(Table::OMEGA, m, tw_l, 0, lo.p, s));
  CHFFT_CUDA(dtype == 0 ? gen_table<float>(Table::OMEGA_STRIDE, m, nhi, tw_l, hi.p, s)
                        : gen_table<double>(Table::OMEGA_STRIDE, m, nhi, tw_l, hi.p, s));
  if (blue) {
    chirp.ensure(n * cb_);
    bhat.ensure(m * cb_);
    CHFFT_CUDA(dtype == 0 ? gen_table<float>(Table::CHIRP, n, n, 0, chirp.p, s)
                          : gen_table<double>(Table::CHIRP, n, n, 0, chirp.p, s));
    // B^ = FFT_M(b) / M computed in FP64 by the four-step f64 engine.
    DevBuf b64, w64;
    b64.ensure(m * sizeof(double2));
    CHFFT_CUDA(gen_table<double>(Table::BLUE_B, n, m, m, b64.p, s));
    BigCore big64;
    if (!big64.build(m, 1, s)) return false;
    w64.ensure(big64.work_elems(1) * sizeof(double2));
    big64.exec(b64.p, b64.p, w64.p, 1, false, 1.0, s);
    if (dtype == 0)
      CHFFT_CUDA(convert_from_f64<float>(static_cast<const double2*>(b64.p), bhat.p, m, s));
    else
      CHFFT_CUDA(cudaMemcpyAsync(bhat.p, b64.p, m * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    CHFFT_CUDA(cudaStreamSynchronize(s));
  }
  return true;
}

FourStep BigCore::fs() const {
  FourStep f{};
  f.n = m;
  f.n1 = n1;
  f.n2 = n2;
  f.tw_shift = tw_shift;
  f.lo = lo.p;
  f.hi = hi.p;
  f.n_user = n;
  f.chirp = chirp.p;
  f.bhat = bhat.p;
  return f;
}

long long BigCore::chunk(long long batch) const {
  // Chunks bound the workspace; within one GB300 the intermediate goes back
  // to HBM whatever the chunk (measured), so few large chunks (few launches,
  // full waves) are fastest.
  long long budget_mb = opts.l2_mb > 0 ? opts.l2_mb : 512;
  if (const char* e = std::getenv("CHFFT_L2_BUDGET_MB")) budget_mb = std::max(1LL, std::atoll(e));
  const long long per = m * (long long)cplx_bytes(dtype) * (blue ? 2 : 1);
  return std::max(1LL, std::min(batch, (budget_mb << 20) / per));
}

// Plus 64 KiB (f32) and one element per transform for the pipelined
// launch's counters (ticket, error word, per-transform tile counts).
long long BigCore::work_elems(long long batch) const {
  long long data = chunk(batch) * m * (blue ? 2 : 1);
  int ring = 0, lead = 0, hints = 0;
  if (pipe_params(batch, &ring, &lead, &hints)) data = std::max(data, (long long)ring * m);
  return data + 8192 + batch;
}

// CHFFT_PIPE: "0" turns the pipelined launch off; "lead,ring,hints" sets its
// schedule (tiles of `lead` transforms' column pass run ahead of the row
// pass, `ring` intermediates, L2 eviction priorities on / off).
bool BigCore::pipe_params(long long batch, int* ring, int* lead, int* hints) const {
  if (!pipe || opts.tc > 0 || batch <= 0) return false;
  int l = 3, r = 6, h = 1;
  if (const char* e = std::getenv("CHFFT_PIPE")) {
    if (e[0] == '0' && e[1] == 0) return false;
    std::sscanf(e, "%d,%d,%d", &l, &r, &h);
  }
  l = (int)std::max<long long>(1, std::min<long long>(l, batch));
  r = std::max(r, l + 1);
  r = (int)std::min<long long>(r, batch);
  *ring = r;
  *lead = l;
  *hints = h;
  return true;
}

void BigCore::exec(const void* in, void* out, void* work, long long batch, bool back, double scale,
                   cudaStream_t s, long long max_chunk, bool library_only) const {
  const size_t cb_ = cplx_bytes(dtype);
  int ring = 0, lead = 0, hints = 0;
  if (!library_only && pipe_params(batch, &ring, &lead, &hints)) {
    // Both passes in one persistent launch (k_pipe.cuh): ring slots of
    // intermediates, then the counters (ticket, error word, tile counts).
    char* ctr = static_cast<char*>(work) + (size_t)ring * m * cb_;
    const size_t ctr_bytes = 16 + 8 * (size_t)batch;
    CHFFT_CUDA(cudaMemsetAsync(ctr, 0, ctr_bytes, s));
    pipe::PipeArgs a{};
    a.out = static_cast<float2*>(out);
    a.ring = static_cast<float2*>(work);
    a.tiles_tw = static_cast<const float2*>(ptw.p);
    a.stw_a = static_cast<const float2*>(pstw_a.p);
    a.stw_b = static_cast<const float2*>(pstw_b.p);
    a.ticket = reinterpret_cast<unsigned long long*>(ctr);
    a.err = reinterpret_cast<int*>(ctr + 8);
    a.sticky = err.dev;
    a.done_a = reinterpret_cast<int*>(ctr + 16);
    a.done_b = a.done_a + batch;
    a.count = batch;
    a.spin_limit = spin_limit();
    a.lead = lead;
    a.ring_slots = ring;
    a.back = back ? 1 : 0;
    a.scale = (float)scale;
    a.hints = hints;
    a.stall = stall_test();
    int ta = 0, tb = 0;
    pipe_tiles(n1, n2, &ta, &tb);
    const long long tasks = batch * (long long)(ta + tb);
    const int grid = (int)std::min<long long>(num_sms(), tasks);
    const int r = pipe_launch(n1, n2, in, a, grid, s);
    if (r == 2) throw Fail{CHFFT_ECUDA, "launch of the pipelined four-step kernel failed"};
    if (r == 0) return;
    // r == 1: the input cannot be described by a tensor map (alignment); the
    // two-launch path below runs instead.
  }
  const long long g = max_chunk > 0 ? std::min(chunk(batch), max_chunk) : chunk(batch);
  char* tmp = static_cast<char*>(work);
  char* tmp2 = tmp + g * m * cb_;
  const FourStep f = fs();
  // f32 tiles of 8 columns / rows: two CTAs per SM (measured faster than 16).
  const int tile_default = opts.fs_tpb > 0 ? opts.fs_tpb : (dtype == 0 ? 8 : 0);
  Geo ga = col_geo(ca, n2, tile_default, opts), gb = col_geo(cb, n1, tile_default, opts);
  const int tc = library_only ? 0 : opts.tc;
  if (tc > 0) {
    // Tile widths the tensor-core kernels take (largest first, from the knob).
    auto tile = [&](const Core& c, Kernel k) {
      for (int t = opts.fs_tpb > 0 ? opts.fs_tpb : 16; t >= 1; t /= 2)
        if (tc_geometry(c, k, t, tc, nullptr)) return t;
      return 0;
    };
    ga.tpb = tile(ca, Kernel::COLS_TW);
    gb.tpb = tile(cb, Kernel::ROWS_T);
    if (!ga.tpb || !gb.tpb)
      throw Fail{CHFFT_EUNSUPPORTED, "tensor-core passes need power-of-two four-step factors >= 16"};
  }
  for (long long c0 = 0; c0 < batch; c0 += g) {
    const long long cnt = std::min(g, batch - c0);
    const char* src = static_cast<const char*>(in) + c0 * n * cb_;
    char* dst = static_cast<char*>(out) + c0 * n * cb_;
    auto pass_a = [&](int mode, const void* i, long long idist, void* o, double sc, int bk) {
      KArgs a{};
      a.core = ca.desc();
      a.tpb = ga.tpb;
      a.ld = ga.ld;
      a.back = bk;
      a.count = cnt;
      a.tiles_per_tr = (n2 + ga.tpb - 1) / ga.tpb;
      a.in = i;
      a.out = o;
      a.scale = sc;
      a.in_dist = idist;
      a.out_dist = m;
      a.ncols = n2;
      launch_pass(true, mode, ca, ga, a, f, (unsigned)(cnt * a.tiles_per_tr), cnt * m, s, library_only, opts.jit, tc);
    };
    auto pass_b = [&](int mode, const void* i, void* o, long long odist, int bk) {
      KArgs a{};
      a.core = cb.desc();
      a.tpb = gb.tpb;
      a.ld = gb.ld;
      a.back = bk;
      a.count = cnt;
      a.tiles_per_tr = (n1 + gb.tpb - 1) / gb.tpb;
      a.in = i;
      a.out = o;
      a.scale = 1.0;
      a.in_dist = m;
      a.out_dist = odist;
      a.ncols = n2;
      launch_pass(false, mode, cb, gb, a, f, (unsigned)(cnt * a.tiles_per_tr), cnt * m, s, library_only, opts.jit, tc);
    };
    if (!blue) {
      pass_a(0, src, n, tmp, scale, back);
      pass_b(0, tmp, dst, n, back);
    } else if (tc <= 0) {
      // Three passes: the inverse FFT is split m = m2 + n2 m1, so its first
      // pass (n2-point FFTs over k2) runs in the forward row pass's CTAs.
      pass_a(1, src, n, tmp, scale, back);  // x c, zero padded
      pass_b(3, tmp, tmp2, m, 0);           // FFT_n2, conj(X B^), FFT_n2, w_M^(k1 m2) -> [m2][k1]
      FourStep fw = f;                      // the last pass sees the n2 x n1 intermediate
      std::swap(fw.n1, fw.n2);
      Geo gc = col_geo(ca, n2, tile_default, opts);
      KArgs a{};
      a.core = ca.desc();
      a.tpb = gc.tpb;
      a.ld = gc.ld;
      a.back = back;
      a.count = cnt;
      a.tiles_per_tr = (n2 + gc.tpb - 1) / gc.tpb;
      a.in = tmp2;
      a.out = dst;
      a.scale = 1.0;
      a.in_dist = m;
      a.out_dist = n;
      a.ncols = n1;
      launch_pass(false, 2, ca, gc, a, fw, (unsigned)(cnt * a.tiles_per_tr), cnt * m, s, library_only, opts.jit, tc);
    } else {
      pass_a(1, src, n, tmp, scale, back);  // x c, zero padded
      pass_b(1, tmp, tmp2, m, 0);           // conj(X B^)
      pass_a(0, tmp2, m, tmp, 1.0, 0);      // inverse FFT as a conjugated forward FFT
      pass_b(2, tmp, dst, n, back);         // conj(.) c, k < n
    }
  }
}

// ---------------------------------------------------------------- cluster latency form

namespace {
// Radix passes of the cluster kernels for a 7-smooth n: radix 4 while
// possible, then 2, 3, 5, 7 (compact bodies: the launch is bound by
// instruction fetch, so few distinct radices). false: not 7-smooth or more
// than 16 passes.
bool cluster_code(long long n, unsigned long long* code, int* np, int* min_r) {
  *code = 0;
  *np = 0;
  *min_r = 8;
  auto push = [&](int r) {
    if (*np >= 16) return false;
    *code |= (unsigned long long)r << (4 * *np);
    ++*np;
    *min_r = std::min(*min_r, r);
    return true;
  };
  while (n % 4 == 0) {
    if (!push(4)) return false;
    n /= 4;
  }
  for (int r : {2, 3, 5, 7})
    while (n % r == 0) {
      if (!push(r)) return false;
      n /= r;
    }
  return n == 1;
}
}  // namespace

bool ClusterCore::build(long long n_, int dtype_, cudaStream_t s, bool beyond_cta) {
  release();
  // CHFFT_CLUSTER: 0 off, 8 or 16 forces the cluster size; unset: the size
  // below. Both dtypes (f32 one-CTA rows are latency-bound at these batches
  // too: N = 1024 12.2 -> 8.1 us, N = 4096 20.4 -> 10.2 us per graph pair,
  // batches 1-9).
  int force = 0;
  if (const char* e = std::getenv("CHFFT_CLUSTER")) {
    if (e[0] == '0' && e[1] == 0) return false;
    force = std::atoi(e);
    if (force != 8 && force != 16) force = 0;
  }
  if (n_ < 64 || n_ > (1LL << 20)) return false;
  // Against the four-step launches (GB300, forward + backward per graph
  // replay): f32 32768 at batches 1-4 32.8 against 36.8-38.9 us but 51
  // against 20 at batch 9, 65536 55 against 34.5; f64 16384 51 against 74
  // at batches 1-4, 96 against 74 at 9, 32768 even. So beyond one CTA the
  // form takes f32 up to 32768 (within the element bound below: 8
  // transforms of 16384, 4 of 32768) and f64 up to 16384, at most 4.
  if (beyond_cta && !force && n_ > (dtype_ == 0 ? 32768 : 16384)) return false;
  const size_t cbytes = cplx_bytes(dtype_);
  struct Pick {
    int n1 = 0, n2 = 0, c = 0, th = 0, lda = 0, ldb = 0, tsz = 0, npa = 0, npb = 0;
    unsigned long long ca = 0, cb = 0;
    size_t smem = 0;
    double cost = 0;
  };
  // 16 CTAs from 1024 points up (measured on GB300, f64 fwd + bwd device
  // time: N = 1024 7.3k against 8.1k cycles per launch, N = 4096 20 against
  // 29 us per pair), 8 below (N = 256: 12 against 14 us).
  const int order[2] = {n_ >= 1024 ? 16 : 8, n_ >= 1024 ? 8 : 16};
  for (int c : order) {
    if (force && c != force) continue;
    Pick best;
    for (long long a1 = c; a1 * c <= n_; a1 += c) {
      if (n_ % a1 || (n_ / a1) % c) continue;
      const long long a2 = n_ / a1;
      Pick q;
      int ra = 0, rb = 0;
      if (!cluster_code(a1, &q.ca, &q.npa, &ra) || !cluster_code(a2, &q.cb, &q.npb, &rb)) continue;
      const int wa = (int)(a2 / c), wb = (int)(a1 / c);
      q.lda = (int)(a1 | 1);
      q.ldb = (int)(a2 | 1);
      q.tsz = std::max(wa * q.lda, wb * q.ldb);
      const size_t tabs = (size_t)(q.npa - 1) * a1 + (size_t)(q.npb - 1) * a2 + (size_t)wa * a1;
      q.smem = (3 * (size_t)q.tsz + tabs) * cbytes + 2 * clus::kClusterMaxPasses * sizeof(clus::FDiv);
      if (q.smem > kMaxSmem) continue;
      // Two threads per element of the CTA's share (n / c), up to the launch bounds.
      const long long per = 2 * n_ / c;
      q.th = (int)std::min<long long>(clus::kClusterThreads, std::max<long long>(32, (per + 31) / 32 * 32));
      // Fewest passes (each a barrier), then the most balanced split.
      q.cost = q.npa + q.npb + 0.01 * std::fabs(std::log2((double)a1 / (double)a2));
      q.n1 = (int)a1;
      q.n2 = (int)a2;
      q.c = c;
      if (!best.c || q.cost < best.cost) best = q;
    }
    if (!best.c) continue;
    const void* k = cluster_kernel(dtype_, best.n1, best.n2, best.c, &best.th);
    if (cluster_max_active(k, best.c, best.th, best.smem) <= 0) continue;
    fn = k;
    n = n_;
    dtype = dtype_;
    n1 = best.n1;
    n2 = best.n2;
    csize = best.c;
    threads = best.th;
    lda = best.lda;
    ldb = best.ldb;
    tsz = best.tsz;
    npa = best.npa;
    npb = best.npb;
    code_a = best.ca;
    code_b = best.cb;
    smem = best.smem;
    // Batches up to 2^18 (f64) or 2^16 (f32) elements, twice that from
    // 8192 points up, at most one transform per SM: measured crossovers
    // against the one-CTA rows (GB300, forward + backward per graph
    // replay): f64 4096 96 against 106 us at batch 76 but 174 against 106
    // at 152, 1024 43 against 55 at 152; f32 4096 20.5 against 20.4 at 38,
    // 1024 14.3 against 14.3 at 76, 256 12.2 against 14.3 at 152. From 8192
    // points the rows take the slower library kernel below 2^18 elements
    // (forward: f32 8192 12.2 against 24.5 us at 16, 16384 18.4 against
    // 32.7 at 8, f64 8192 88 against 108 at 64), so the cluster keeps the
    // batches up to half that; f32 within one CTA up to just below it
    // (the cluster at 32 x 8192 takes 16.3 us, the library rows 24.5).
    // CHFFT_CLUSTER_MAX_BATCH overrides.
    long long elems = (dtype_ == 0 ? (1LL << 16) : (1LL << 18)) << (n_ >= 8192 ? 1 : 0);
    if (dtype_ == 0 && !beyond_cta && n_ >= 8192) elems = (1LL << 18) - 1;  // want_specialised's bound
    max_batch = std::max<long long>(1, std::min<long long>(num_sms(), elems / n_));
    if (beyond_cta && dtype_ != 0) max_batch = std::min<long long>(max_batch, 4);
    if (const char* e = std::getenv("CHFFT_CLUSTER_MAX_BATCH")) max_batch = std::max(0LL, std::atoll(e));
    tab_a.ensure(std::max<size_t>(1, (size_t)(npa - 1) * n1) * cbytes);
    tab_b.ensure(std::max<size_t>(1, (size_t)(npb - 1) * n2) * cbytes);
    CHFFT_CUDA(cluster_pass_tables(dtype, n1, code_a, npa, tab_a.p, s));
    CHFFT_CUDA(cluster_pass_tables(dtype, n2, code_b, npb, tab_b.p, s));
    // The scales of the CFft1D methods, computed as the plan computes them.
    scales[0] = 1.0;
    scales[1] = 1.0 / std::sqrt((double)n);
    scales[2] = 1.0 / (double)n;
    for (int k = 0; k < kScales; k++) {
      blk[k].ensure((size_t)n * cbytes);
      CHFFT_CUDA(cluster_block_table(dtype, n, n1, scales[k], blk[k].p, s));
    }
    err.ensure();
    return true;
  }
  return false;
}

bool ClusterCore::exec(const void* in, void* out, long long batch, bool back, double scale, cudaStream_t s) const {
  int k = 0;
  while (k < kScales && scales[k] != scale) k++;
  if (k == kScales) return false;
  clus::ClusterArgs a{};
  a.in = in;
  a.out = out;
  a.tab_a = tab_a.p;
  a.tab_b = tab_b.p;
  a.blk = blk[k].p;
  a.dist = n;
  a.code_a = code_a;
  a.code_b = code_b;
  a.npa = npa;
  a.npb = npb;
  a.n1 = n1;
  a.n2 = n2;
  a.wa = n2 / csize;
  a.wb = n1 / csize;
  a.lda = lda;
  a.ldb = ldb;
  a.tsz = tsz;
  // Divisions by each pass's Ns (the product of the earlier radices) and by
  // the columns / rows per CTA.
  auto mk_div = [](int d) {
    clus::FDiv f;
    f.d = d;
    f.m = ((1ULL << 40) / (unsigned long long)d) + 1;
    return f;
  };
  for (int pass = 0, ns = 1; pass < npa; ns *= (int)((code_a >> (4 * pass)) & 15), pass++) a.ns_a[pass] = mk_div(ns);
  for (int pass = 0, ns = 1; pass < npb; ns *= (int)((code_b >> (4 * pass)) & 15), pass++) a.ns_b[pass] = mk_div(ns);
  a.div_wa = mk_div(n2 / csize);
  a.div_wb = mk_div(n1 / csize);
  a.back = back ? 1 : 0;
  a.err = err.dev;
  a.spin_limit = spin_limit();
  a.stall = stall_test();
  CHFFT_CUDA(cluster_launch(fn, a, batch, csize, threads, smem, s));
  return true;
}

}  // namespace chfft
