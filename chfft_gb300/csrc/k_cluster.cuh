// Latency form of a small batch: one transform of length N = N1 x N2 spread
// over a thread-block cluster of C CTAs (C = 8 or 16, one CTA per SM), the
// four-step exchange through distributed shared memory.
//
// A single f64 transform in one CTA is bound by that SM's FP64 rate (about
// two FMAs per clock on GB300: a 1024-point FFT is several microseconds of
// FP64 issue alone); spread over the cluster each SM does 1/C of it:
//   pass A: CTA c takes the columns n2 in [c WA, (c+1) WA), WA = N2 / C,
//           runs their N1-point FFTs and keeps the result in its own shared
//           memory, column t at t * lda;
//   cluster barrier (release / acquire: every CTA's result visible
//           cluster-wide);
//   pass B: CTA c takes the rows k1 in [c WB, (c+1) WB), WB = N1 / C, reads
//           element (k1, n2) from CTA n2 / WA (a shared-memory address of
//           that CTA, mapa), multiplies it by w_N^(k1 n2), runs the N2-point
//           FFTs and stores X[k1 + N1 k2];
//   cluster arrive after the reads of pass B, wait before exit (no CTA
//           exits while the others may still read its shared memory).
// Every read of the input precedes the first barrier and every write of the
// output follows it, so in-place calls are safe. The backward transform
// conjugates on the way in and out and the scale applies on load, as the
// row kernels do (chfft's out-of-place gather scales on load,
// src/mixed_radix.rs:32-43). The four-step factorisation is the one the
// reference's mixed-radix DIT computes with its precomputed twiddles
// (src/mixed_radix.rs:60-166): X[k1 + N1 k2] = sum_n2 w_N2^(n2 k2)
// w_N^(n2 k1) sum_n1 x[n2 + N2 n1] w_N1^(n1 k1).
#pragma once

#include "kernels.cuh"

namespace chfft {
namespace clus {

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cluster_size() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_arrive() {
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() {
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_sync() {
  cluster_arrive();
  cluster_wait();
}
// Generic address of the same shared-memory location in CTA `rank` of the cluster.
template <typename P>
__device__ __forceinline__ P* peer(P* local, unsigned rank) {
  unsigned long long out;
  asm volatile("mapa.u64 %0, %1, %2;" : "=l"(out) : "l"(reinterpret_cast<unsigned long long>(local)), "r"(rank));
  return reinterpret_cast<P*>(out);
}
// Programmatic dependent launch: the next kernel on the stream may start
// its prologue now; this kernel's reads of memory an earlier kernel wrote
// wait for that kernel's completion (no-ops without the launch attribute).
__device__ __forceinline__ void allow_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void wait_prerequisites() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ unsigned su32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
// Shared::cluster address of the same location in CTA `rank`.
__device__ __forceinline__ unsigned peer_u32(unsigned local, unsigned rank) {
  unsigned out;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(out) : "r"(local), "r"(rank));
  return out;
}
__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// The phase's one arrival, expecting `bytes` of remote stores.
__device__ __forceinline__ void mbar_arrive_expect(unsigned long long* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(su32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Store to another CTA's shared memory that counts its bytes on that CTA's mbarrier.
__device__ __forceinline__ void st_async(unsigned addr, double v, unsigned bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.f64 [%0], %1, [%2];" ::"r"(addr), "d"(v), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void st_async(unsigned addr, float v, unsigned bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.f32 [%0], %1, [%2];" ::"r"(addr), "f"(v), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void prefetch_l1(const void* p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

// Threads per CTA at most (the launch bounds).
constexpr int kClusterThreads = 512;
constexpr int kClusterMaxPasses = 16;

// Division by a run-time divisor d < 2^19 of numerators x < 2^21 as one
// wide multiply: q = (x * m) >> 40, m = floor(2^40 / d) + 1. With
// e = m d - 2^40 in (0, d], x e < 2^40 keeps x e / (d 2^40) below 1 / d,
// the smallest gap between x / d and the next integer, so q = floor(x / d).
struct FDiv {
  unsigned long long m;
  int d;
};
__device__ __forceinline__ int fdiv(int x, const FDiv& f) {
  return (int)(((unsigned long long)(unsigned)x * f.m) >> 40);
}

// Sign flips and component selects on the integer pipe (GB300's FP64 pipe
// issues one warp instruction per 64 cycles per SM sub-partition; a
// negation there would cost as much as an add).
__device__ __forceinline__ double flip(double v) {
  return __hiloint2double(__double2hiint(v) ^ (int)0x80000000, __double2loint(v));
}
__device__ __forceinline__ float flip(float v) { return __int_as_float(__float_as_int(v) ^ (int)0x80000000); }
template <typename R>
__device__ __forceinline__ R flip_if(R v, bool n) {
  return n ? flip(v) : v;
}
template <typename C>
__device__ __forceinline__ C conj_if(C v, bool n) {
  return n ? mk(v.x, flip(v.y)) : v;
}
template <typename C>
__device__ __forceinline__ typename Real<C>::type comp(const C& v, int h) {
  return h ? v.y : v.x;
}

// FP64 issue. On GB300 a warp instruction on the FP64 pipe occupies its
// sub-partition for about 64 cycles whatever the active lanes (measured: a
// CTA of one warp spends ~2000 cycles per radix-4 pass of 28 FP64
// instructions per thread; half a warp takes as long), so a small f64
// transform is bound by the FP64 instructions on each thread's chain, and
// the shape that minimises them puts one thread on each HALF element, one
// warp per sub-partition:
//  * a thread pair computes ONE output of a radix-R butterfly, lane parity
//    h taking its real (h = 0) or imaginary (h = 1) part (radix 4: three
//    adds, the k-dependent signs and the -i rotation as integer selects);
//  * the twiddle of the next pass's input is multiplied into the output by
//    its producer (a table per pass: the pair swaps parts with one shuffle,
//    then two FP64 instructions each), the four-step twiddle (the method's
//    scale folded in) by the last pass of the columns;
//  * passes ping-pong between shared-memory buffers (one barrier each);
//    the columns' last pass stores each output straight into the shared
//    memory of the CTA whose rows hold it (st.async, each store counting
//    its bytes on that CTA's mbarrier: a CTA starts its rows when all its
//    bytes have landed, with no cluster-wide barrier), so the rows run on
//    local data and the last pass stores to global memory.
// A 1024-point transform on 16 CTAs of 128 threads is then 25 FP64
// instructions per thread (the engine's row kernel: ~1100 per warp).
struct ClusterArgs {
  const void* in;
  void* out;
  const void* tab_a;        // per-pass output twiddles of the n1-point FFT: (npa - 1) x n1
  const void* tab_b;        // per-pass output twiddles of the n2-point FFT: (npb - 1) x n2
  const void* blk;          // four-step twiddles x scale, CTA c's block at c * wa * n1: [t][k1]
  long long dist;           // elements between transforms (input and output)
  unsigned long long code_a, code_b;  // radix of pass p at bits [4p, 4p + 4)
  FDiv ns_a[kClusterMaxPasses], ns_b[kClusterMaxPasses];  // divisions by Ns of each pass
  FDiv div_wa, div_wb;
  int npa, npb;             // passes of the n1- and n2-point FFTs
  int n1, n2, wa, wb;       // wa = n2 / C columns, wb = n1 / C rows per CTA
  int lda, ldb, tsz;        // sequence strides; elements per buffer
  int back;
  int* err;                 // host-mapped error word (a bounded wait gave up: 7), may be null
  long long spin_limit;     // polls of the rows' arrival wait before it gives up
  int stall;                // test hook: expect 16 bytes that never come, so the wait runs out
};

// Part h (0 real, 1 imaginary) of output k of a forward radix-R DFT of v.
template <int R, typename C>
__device__ __forceinline__ typename Real<C>::type dft_part(const C* v, int k, int h) {
  using Rl = typename Real<C>::type;
  if constexpr (R == 2) {
    return comp(v[0], h) + flip_if(comp(v[1], h), k != 0);
  } else if constexpr (R == 4) {
    // X_k = (v0 +- v2) + [(-i) if k odd] (v1 +- v3) x (+-1 for k >= 2);
    // (-i) b has parts (b.y, -b.x).
    const bool odd = (k & 1) != 0;
    const Rl a = comp(v[0], h) + flip_if(comp(v[2], h), odd);
    const int hb = odd ? 1 - h : h;
    const Rl b = comp(v[1], hb) + flip_if(comp(v[3], hb), odd);
    return a + flip_if(b, (odd && h == 1) != ((k & 2) != 0));
  } else {
    // Odd prime R: pairs (r, R - r) give (v_r + v_{R-r}) cos(2 pi r k / R)
    // - i (v_r - v_{R-r}) sin(2 pi r k / R); -i d has parts (d.y, -d.x).
    Rl x = comp(v[0], h);
#pragma unroll
    for (int r = 1; r <= (R - 1) / 2; r++) {
      const Rl t = comp(v[r], h) + comp(v[R - r], h);
      const Rl d = comp(v[r], 1 - h) - comp(v[R - r], 1 - h);
      const int m = (r * k) % R;
      Rl c = Rl(1), sn = Rl(0);
#pragma unroll
      for (int q = 1; q < R; q++)
        if (m == q) {
          c = Rl(ct::cos2pi(q, R));
          sn = Rl(ct::sin2pi(q, R));
        }
      x = fma(c, t, x);
      x = fma(flip_if(sn, h == 1), d, x);
    }
    return x;
  }
}

// Where a pass writes.
enum { kToSmemNext = 0, kToPeers = 1, kToGlobal = 2 };

struct PassGeo {
  int n, tpb, ld;  // sequence length, sequences, stride
  FDiv dt;         // division by tpb
};

// One radix-R Stockham pass. Work item w = 2 e + h: part h of output
// element e = t + tpb * pos (t fastest, odd strides, distinct banks);
// pos = q Ns R + k Ns + jm reads the butterfly j = q Ns + jm inputs
// j + r n / R. Every lane of a warp runs every trip (a lane past the end
// computes on element 0 and stores nothing), so the pair shuffle sees
// full warps. OUT: kToSmemNext multiplies by tw[pos] (the next pass's
// input twiddle); kToPeers multiplies by tw[t * n + pos] (the four-step
// block) and stores element (k1 = pos, column col0 + t) into dst of CTA
// k1 / wb, row k1 mod wb, counted on that CTA's barrier `bar`;
// kToGlobal stores X[off + t + n1 pos] (conjugated for the backward
// transform).
template <int R, int OUT, typename C>
__device__ __forceinline__ void epass(const PassGeo& g, const FDiv& ns, const C* src, C* dst, const C* tw,
                                      const ClusterArgs& a, int col0, C* out, unsigned long long* bar) {
  using Rl = typename Real<C>::type;
  const int nb = g.n / R, total = 2 * g.tpb * g.n, Ns = ns.d;
  const int h = threadIdx.x & 1;
  for (int base = 0; base < total; base += blockDim.x) {
    const int w = base + threadIdx.x;
    const bool act = w < total;
    const int e = act ? w >> 1 : 0;
    const int pos = fdiv(e, g.dt), t = e - pos * g.tpb;
    const int u = fdiv(pos, ns), jm = pos - u * Ns;
    const int q = u / R, k = u - q * R;
    const C* s = src + t * g.ld + q * Ns + jm;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = s[r * nb];
    const Rl x = dft_part<R>(v, k, h);
    if constexpr (OUT == kToGlobal) {
      if (act) reinterpret_cast<Rl*>(out)[2 * ((long long)t + (long long)a.n1 * pos) + h] = flip_if(x, a.back && h);
    } else {
      // (x_re + i x_im)(w_re + i w_im): part h = x_h w_re -+ x_{1-h} w_im.
      const Rl other = __shfl_xor_sync(0xffffffffu, x, 1);
      const C wv = OUT == kToSmemNext ? tw[pos] : tw[t * g.n + pos];
      const Rl y = fma(x, wv.x, flip_if(other * wv.y, h == 0));
      if constexpr (OUT == kToSmemNext) {
        if (act) reinterpret_cast<Rl*>(dst)[2 * (t * g.ld + pos) + h] = y;
      } else {
        const int owner = fdiv(pos, a.div_wb), tb = pos - owner * a.wb;
        const unsigned la = su32(reinterpret_cast<Rl*>(dst) + 2 * (tb * a.ldb + col0 + t) + h);
        if (act) st_async(peer_u32(la, (unsigned)owner), y, peer_u32(su32(bar), (unsigned)owner));
      }
    }
  }
}

template <int OUT, typename C>
__device__ __forceinline__ void epass_r(int R, const PassGeo& g, const FDiv& ns, const C* src, C* dst, const C* tw,
                                        const ClusterArgs& a, int col0, C* out, unsigned long long* bar = nullptr) {
  switch (R) {
    case 4: epass<4, OUT>(g, ns, src, dst, tw, a, col0, out, bar); break;
    case 2: epass<2, OUT>(g, ns, src, dst, tw, a, col0, out, bar); break;
    case 3: epass<3, OUT>(g, ns, src, dst, tw, a, col0, out, bar); break;
    case 5: epass<5, OUT>(g, ns, src, dst, tw, a, col0, out, bar); break;
    case 7: epass<7, OUT>(g, ns, src, dst, tw, a, col0, out, bar); break;
    default: break;
  }
}

// Grid: C CTAs per transform in clusters of C (launch attribute). Dynamic
// shared memory: three buffers of tsz elements (the columns ping-pong the
// first two; the third receives this CTA's rows from every CTA's last
// column pass, and the rows ping-pong it with the first), the per-pass
// twiddle tables of both FFTs, this CTA's four-step block, then the
// per-pass divisions. Launched with programmatic stream serialisation: the
// next kernel's CTAs may start while this one runs, and every read of the
// input waits for the kernels before it (griddepcontrol). Synchronisation:
// each CTA initialises its arrival
// mbarrier (one arrival expecting its rows' bytes) and arrives on the
// cluster barrier at entry; the barrier is waited for before the first
// remote store (every CTA of the cluster has started and initialised its
// mbarrier); the rows start when their bytes have landed (a bounded wait:
// on time-out the error word gets 7 and the CTA runs on, in bounds).
template <typename T>
__global__ void __launch_bounds__(kClusterThreads, 1) k_c2c_cluster(const ClusterArgs a) {
  using C = cx_t<T>;
  constexpr int kU = 4;  // loads in flight per thread before their stores
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long arrived;
  if (threadIdx.x == 0) {
    mbar_init(&arrived, 1);
    mbar_arrive_expect(&arrived, (unsigned)(a.wb * a.n2 * sizeof(C)) + (a.stall ? 16u : 0u));
  }
  allow_dependents();
  cluster_arrive();
  const unsigned c = cluster_rank();
  const long long tr = blockIdx.x / cluster_size();
  const int n1 = a.n1, n2 = a.n2, wa = a.wa, wb = a.wb;
  const int ta_n = (a.npa - 1) * n1, tb_n = (a.npb - 1) * n2, blk_n = wa * n1;
  C* buf0 = reinterpret_cast<C*>(smem_raw);
  C* buf1 = buf0 + a.tsz;
  C* buf2 = buf1 + a.tsz;
  C* sta = buf2 + a.tsz;
  C* stb = sta + ta_n;
  C* sblk = stb + tb_n;
  FDiv* nsd = reinterpret_cast<FDiv*>(sblk + blk_n);  // ns_a then ns_b
  // Tables, divisions and columns [c wa, (c+1) wa) of the input (element
  // (i, t) at in[i n2 + c wa + t] into buf0[t lda + i], conjugated for the
  // backward transform), every load issued before the stores.
  {
    const C* ga = static_cast<const C*>(a.tab_a);
    const C* gb = static_cast<const C*>(a.tab_b);
    const C* gk = static_cast<const C*>(a.blk) + (size_t)c * blk_n;
    const int ntab = ta_n + tb_n + blk_n;
    if (threadIdx.x < 2 * kClusterMaxPasses)
      nsd[threadIdx.x] = threadIdx.x < kClusterMaxPasses ? a.ns_a[threadIdx.x] : a.ns_b[threadIdx.x - kClusterMaxPasses];
    const C* in = static_cast<const C*>(a.in) + tr * a.dist + (long long)c * wa;
    const int tot = n1 * wa;
    const int steps = max(tot, ntab);
    wait_prerequisites();
    for (int b0 = threadIdx.x; b0 < steps; b0 += kU * blockDim.x) {
      C v[kU], w[kU];
#pragma unroll
      for (int u = 0; u < kU; u++) {
        const int b = b0 + u * blockDim.x;
        if (b < tot) {
          const int i = fdiv(b, a.div_wa), t = b - i * wa;
          v[u] = in[(long long)i * n2 + t];
        }
        if (b < ntab) w[u] = b < ta_n ? ga[b] : b < ta_n + tb_n ? gb[b - ta_n] : gk[b - ta_n - tb_n];
      }
#pragma unroll
      for (int u = 0; u < kU; u++) {
        const int b = b0 + u * blockDim.x;
        if (b < tot) {
          const int i = fdiv(b, a.div_wa), t = b - i * wa;
          buf0[t * a.lda + i] = conj_if(v[u], a.back != 0);
        }
        if (b < ntab) sta[b] = w[u];
      }
    }
  }
  __syncthreads();
  // Columns: n1-point FFTs of the wa sequences; the last pass multiplies by
  // the four-step block and stores into the rows' owners.
  {
    C* src = buf0;
    C* dst = buf1;
    const PassGeo g{n1, wa, a.lda, a.div_wa};
#pragma unroll 1
    for (int p = 0; p + 1 < a.npa; p++) {
      const int R = (int)((a.code_a >> (4 * p)) & 15);
      epass_r<kToSmemNext>(R, g, nsd[p], src, dst, sta + p * n1, a, 0, (C*)nullptr);
      __syncthreads();
      C* t = src;
      src = dst;
      dst = t;
    }
    cluster_wait();  // every CTA of the cluster has started
    const int R = (int)((a.code_a >> (4 * (a.npa - 1))) & 15);
    epass_r<kToPeers>(R, g, nsd[a.npa - 1], src, buf2, sblk, a, (int)c * wa, (C*)nullptr, &arrived);
  }
  // Every CTA's rows are in its buf2 once their bytes have landed.
  for (long long i = 0; !mbar_test(&arrived, 0); i++) {
    if (i >= a.spin_limit) {
      if (a.err && threadIdx.x == 0) {
        *(volatile int*)a.err = 7;
        __threadfence_system();
      }
      break;
    }
  }
  // Rows k1 = r0 + t: n2-point FFTs, the last pass storing X[k1 + n1 k2].
  {
    const int r0 = (int)c * wb;
    C* out = static_cast<C*>(a.out) + tr * a.dist + r0;
    const PassGeo g{n2, wb, a.ldb, a.div_wb};
    const FDiv* nsb = nsd + kClusterMaxPasses;
    C* src = buf2;
    C* dst = buf0;
#pragma unroll 1
    for (int p = 0; p + 1 < a.npb; p++) {
      const int R = (int)((a.code_b >> (4 * p)) & 15);
      epass_r<kToSmemNext>(R, g, nsb[p], src, dst, stb + p * n2, a, 0, out);
      __syncthreads();
      src = dst;
      dst = src == buf0 ? buf1 : buf0;
    }
    const int R = (int)((a.code_b >> (4 * (a.npb - 1))) & 15);
    epass_r<kToGlobal>(R, g, nsb[a.npb - 1], src, dst, stb, a, 0, out);
  }
}

// ---------------------------------------------------------------------------
// The same kernel with the split fixed at compile time, for the power-of-two
// splits the plans pick (N = 64 .. 16384): every division, stride and pass
// radix is a constant, the passes are straight-line code and each thread's
// items of a pass are unrolled together, so the index arithmetic that
// dominates the run-time-shape kernel's pass latency folds away. Shared
// memory layout, tables and arguments are the run-time kernel's.
CHFFT_HD constexpr int pow2_passes(int n) {  // radix 4 while possible, then 2
  int p = 0;
  while (n % 4 == 0) {
    n /= 4;
    p++;
  }
  return n == 2 ? p + 1 : p;
}
CHFFT_HD constexpr int pow2_radix(int n, int p) {
  int q4 = 0;
  while (n % 4 == 0) {
    n /= 4;
    q4++;
  }
  return p < q4 ? 4 : 2;
}
CHFFT_HD constexpr int pow2_ns(int n, int p) {
  int s = 1;
  for (int i = 0; i < p; i++) s *= pow2_radix(n, i);
  return s;
}

template <int N1, int N2, int CS>
struct CShape {
  static constexpr int WA = N2 / CS, WB = N1 / CS;
  static constexpr int LDA = N1 | 1, LDB = N2 | 1;
  static constexpr int TSZ = WA * LDA > WB * LDB ? WA * LDA : WB * LDB;
  static constexpr int E = N1 * WA;  // elements per CTA in either phase
  static constexpr int THREADS = 2 * E < 32 ? 32 : (2 * E > kClusterThreads ? kClusterThreads : 2 * E);
  static constexpr int NPA = pow2_passes(N1), NPB = pow2_passes(N2);
  static_assert(N1 % CS == 0 && N2 % CS == 0, "split not divisible by the cluster size");
};

// One compile-time radix-R pass: ITEMS = 2 TPB N work items over THREADS
// threads, every thread running every trip (the pair shuffle sees full
// warps), a trip's items unrolled together.
template <int R, int NS, int N, int TPB, int LD, int OUT, int THREADS, int WB, int LDB, int N1, typename C>
__device__ __forceinline__ void spass(const C* src, C* dst, const C* tw, const ClusterArgs& a, int col0, C* out,
                                      unsigned long long* bar) {
  using Rl = typename Real<C>::type;
  constexpr int NB = N / R, ITEMS = 2 * TPB * N, TRIPS = (ITEMS + THREADS - 1) / THREADS;
  const int h = threadIdx.x & 1;
#pragma unroll
  for (int it = 0; it < TRIPS; it++) {
    const int w = it * THREADS + threadIdx.x;
    const bool act = ITEMS % THREADS == 0 || w < ITEMS;
    const int e = act ? w >> 1 : 0;
    const int pos = e / TPB, t = e % TPB;
    const int u = pos / NS, jm = pos % NS;
    const int q = u / R, k = u % R;
    const C* s = src + t * LD + q * NS + jm;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = s[r * NB];
    const Rl x = dft_part<R>(v, k, h);
    if constexpr (OUT == kToGlobal) {
      if (act) reinterpret_cast<Rl*>(out)[2 * (t + N1 * pos) + h] = flip_if(x, a.back && h);
    } else {
      const Rl other = __shfl_xor_sync(0xffffffffu, x, 1);
      const C wv = OUT == kToSmemNext ? tw[pos] : tw[t * N + pos];
      const Rl y = fma(x, wv.x, flip_if(other * wv.y, h == 0));
      if constexpr (OUT == kToSmemNext) {
        if (act) reinterpret_cast<Rl*>(dst)[2 * (t * LD + pos) + h] = y;
      } else {
        const int owner = pos / WB, tb = pos % WB;
        const unsigned la = su32(reinterpret_cast<Rl*>(dst) + 2 * (tb * LDB + col0 + t) + h);
        if (act) st_async(peer_u32(la, (unsigned)owner), y, peer_u32(su32(bar), (unsigned)owner));
      }
    }
  }
}

template <int P, class S, int N1, int N2, typename C>
__device__ __forceinline__ void scols(C* src, C* dst, C* buf2, const C* sta, const C* sblk, const ClusterArgs& a,
                                      int col0, unsigned long long* bar) {
  constexpr int R = pow2_radix(N1, P), NS = pow2_ns(N1, P);
  if constexpr (P + 1 < S::NPA) {
    spass<R, NS, N1, S::WA, S::LDA, kToSmemNext, S::THREADS, S::WB, S::LDB, N1>(src, dst, sta + P * N1, a, col0,
                                                                             (C*)nullptr, bar);
    __syncthreads();
    scols<P + 1, S, N1, N2>(dst, src, buf2, sta, sblk, a, col0, bar);
  } else {
    cluster_wait();  // every CTA of the cluster has started
    spass<R, NS, N1, S::WA, S::LDA, kToPeers, S::THREADS, S::WB, S::LDB, N1>(src, buf2, sblk, a, col0, (C*)nullptr,
                                                                          bar);
  }
}

template <int P, class S, int N1, int N2, typename C>
__device__ __forceinline__ void srows(C* src, C* dst, C* other, const C* stb, const ClusterArgs& a, C* out) {
  constexpr int R = pow2_radix(N2, P), NS = pow2_ns(N2, P);
  if constexpr (P + 1 < S::NPB) {
    spass<R, NS, N2, S::WB, S::LDB, kToSmemNext, S::THREADS, S::WB, S::LDB, N1>(src, dst, stb + P * N2, a, 0, out,
                                                                             nullptr);
    __syncthreads();
    srows<P + 1, S, N1, N2>(dst, other, dst, stb, a, out);
  } else {
    spass<R, NS, N2, S::WB, S::LDB, kToGlobal, S::THREADS, S::WB, S::LDB, N1>(src, dst, stb, a, 0, out, nullptr);
  }
}

template <typename T, int N1, int N2, int CS>
__global__ void __launch_bounds__(CShape<N1, N2, CS>::THREADS, 1) k_c2c_cluster_s(const ClusterArgs a) {
  using C = cx_t<T>;
  using S = CShape<N1, N2, CS>;
  constexpr int TA = (S::NPA - 1) * N1, TB = (S::NPB - 1) * N2, BLK = S::WA * N1, NTAB = TA + TB + BLK;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long arrived;
  if (threadIdx.x == 0) {
    mbar_init(&arrived, 1);
    mbar_arrive_expect(&arrived, (unsigned)(S::WB * N2 * sizeof(C)) + (a.stall ? 16u : 0u));
  }
  allow_dependents();
  cluster_arrive();
  const unsigned c = cluster_rank();
  const long long tr = blockIdx.x / CS;
  C* buf0 = reinterpret_cast<C*>(smem_raw);
  C* buf1 = buf0 + S::TSZ;
  C* buf2 = buf1 + S::TSZ;
  C* sta = buf2 + S::TSZ;
  C* stb = sta + TA;
  C* sblk = stb + TB;
  {
    const C* ga = static_cast<const C*>(a.tab_a);
    const C* gb = static_cast<const C*>(a.tab_b);
    const C* gk = static_cast<const C*>(a.blk) + (size_t)c * BLK;
    const C* in = static_cast<const C*>(a.in) + tr * a.dist + (long long)c * S::WA;
    constexpr int STEPS = (S::E > NTAB ? S::E : NTAB), TRIPS = (STEPS + S::THREADS - 1) / S::THREADS;
    C v[TRIPS], w[TRIPS];
    // The plan's tables first (no earlier kernel writes them), then the
    // input once the kernels it depends on have completed.
#pragma unroll
    for (int u = 0; u < TRIPS; u++) {
      const int b = u * S::THREADS + threadIdx.x;
      if (b < NTAB) w[u] = b < TA ? ga[b] : b < TA + TB ? gb[b - TA] : gk[b - TA - TB];
    }
    wait_prerequisites();
#pragma unroll
    for (int u = 0; u < TRIPS; u++) {
      const int b = u * S::THREADS + threadIdx.x;
      if (b < S::E) v[u] = in[(long long)(b / S::WA) * N2 + b % S::WA];
    }
#pragma unroll
    for (int u = 0; u < TRIPS; u++) {
      const int b = u * S::THREADS + threadIdx.x;
      if (b < S::E) buf0[(b % S::WA) * S::LDA + b / S::WA] = conj_if(v[u], a.back != 0);
      if (b < NTAB) sta[b] = w[u];
    }
  }
  __syncthreads();
  scols<0, S, N1, N2>(buf0, buf1, buf2, sta, sblk, a, (int)c * S::WA, &arrived);
  for (long long i = 0; !mbar_test(&arrived, 0); i++) {
    if (i >= a.spin_limit) {
      if (a.err && threadIdx.x == 0) {
        *(volatile int*)a.err = 7;
        __threadfence_system();
      }
      break;
    }
  }
  srows<0, S, N1, N2>(buf2, buf0, buf1, stb, a, static_cast<C*>(a.out) + tr * a.dist + (int)c * S::WB);
}

}  // namespace clus
}  // namespace chfft
