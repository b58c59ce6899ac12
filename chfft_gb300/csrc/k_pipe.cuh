// Pipelined four-step: both passes of a batched f32 FFT of length
// N = N1 x N2 (N1, N2 in {256, 512, 1024}) in one persistent launch.
//
// chfft runs such a length as log_4 N radix-4 passes over the whole array
// (src/mixed_radix.rs:104-166, :230-270), each one a strided sweep through
// memory. Here the FFT is split four-step, x[n1 N2 + n2]:
//   pass A: for each column n2, an N1-point FFT over n1, times w_N^(k1 n2),
//           written in place order to an intermediate T[k1][n2];
//   pass B: for each row k1 of T, an N2-point FFT over n2, written
//           transposed to X[k1 + N1 k2].
// Both passes are tiles of 64 KiB (pass A: WA = 8192 / N1 adjacent columns,
// pass B: WB = 8192 / N2 adjacent rows), and one launch of one CTA per SM
// runs every tile of both passes:
//   - a producer thread takes tiles from a ticket counter in the order
//     A(0..lead-1), then A(k+lead), B(k) for k = 0, 1, ..., waits until a
//     tile's inputs exist (B(k): every A(k) tile done; A(k): every
//     B(k-ring) tile done, whose ring slot it overwrites), and loads the tile
//     into one of two shared-memory stages with the tensor memory accelerator
//     (pass A: a 2-D tensor map over the input, boxes of WA x 256, plus the
//     tile's twiddle tables; pass B: one bulk copy of WB contiguous rows of
//     T), completing on an mbarrier;
//   - eight consumer warps run the tile's two radix passes (an N/32-point
//     pass, then a radix-32 pass) through a padded exchange buffer and store
//     to global memory, while the producer already loads the next tile;
//   - the intermediate of transform k lives in ring slot k % ring, a few
//     transforms' worth (tens of MiB), so pass B finds it in L2 and HBM sees
//     one read of the input and one write of the output.
// A CTA only waits on tiles whose tickets were taken earlier, by CTAs that
// are running, so no order of CTA residency can deadlock. Every wait is
// bounded: on time-out a CTA records an error code (device word, plus the
// plan's host-mapped word) and the launch winds down without hanging.
#pragma once

#include "kernels.cuh"

namespace chfft {
namespace pipe {

// CUtensorMap's layout: 128 opaque bytes, 64-byte aligned.
struct alignas(64) TensorMap {
  unsigned long long opaque[16];
};

struct PipeArgs {
  float2* out;              // count transforms of N, natural order
  float2* ring;             // ring_slots intermediates of N
  const float2* tiles_tw;   // per pass-A tile: atab[32][WA] then wtab[N1/32][WA] (pipe_twiddles)
  const float2* stw_a;      // stage twiddles of the N1-point FFT, pass order (N1/32, 32)
  const float2* stw_b;      // the same for N2
  unsigned long long* ticket;
  int* err;                 // this launch's error word (zeroed with the counters)
  int* sticky;              // host-mapped error word of the plan, may be null
  int* done_a;              // per transform: finished pass-A tiles
  int* done_b;              // per transform: finished pass-B tiles
  long long count;          // transforms
  long long spin_limit;     // polls (~0.25 us apart) before a wait gives up
  int lead, ring_slots;
  int back;                 // backward transform (conjugate in and out)
  float scale;
  int hints;                // L2 eviction priorities: input / output first, ring last
  int stall;                // test hook: > 0 makes B(0)'s dependency unreachable
};

constexpr int kConsumers = 256;  // eight consumer warps
constexpr int kConsumerWarps = kConsumers / 32;
constexpr int kThreads = 320;    // plus the producer warp and the reporter warp
constexpr int kTileElems = 8192; // complex elements per tile (64 KiB)

// Exchange-buffer stride: >= n + n/32 (one pad slot per 32 elements) and
// congruent to q mod 2q, q = 16 / w, so the w sequences x 32/w elements a
// warp touches fall in distinct bank pairs.
__host__ __device__ constexpr int xch_ld(int n, int w) {
  const int q = w >= 16 ? 1 : 16 / w;
  int ld = n + n / 32;
  while (ld % (2 * q) != q) ld++;
  return ld;
}
__host__ __device__ constexpr int xch_pad(int i) { return i + (i >> 5); }

template <int N1, int N2>
struct Shape {
  static constexpr int N = N1 * N2;
  static constexpr int WA = kTileElems / N1;  // columns per pass-A tile
  static constexpr int WB = kTileElems / N2;  // rows per pass-B tile
  static constexpr int TA = N2 / WA;          // pass-A tiles per transform
  static constexpr int TB = N1 / WB;          // pass-B tiles per transform
  static constexpr int BOXR = N1 < 256 ? N1 : 256;  // rows per tensor-map box
  static constexpr int LDA = xch_ld(N1, WA);
  static constexpr int LDB = xch_ld(N2, WB);
  static constexpr int XCH = (WA * LDA > WB * LDB ? WA * LDA : WB * LDB);
  // shared-memory carve-up (bytes from a 1024-aligned base)
  static constexpr int OFF_XCH = 2 * kTileElems * 8;
  static constexpr int OFF_STWA = OFF_XCH + ((XCH * 8 + 127) / 128) * 128;
  static constexpr int NSTWA = 31 * (N1 / 32);
  static constexpr int NSTWB = 31 * (N2 / 32);
  static constexpr int OFF_STWB = OFF_STWA + ((NSTWA * 8 + 127) / 128) * 128;
  // stage twiddles of N2 (absent when N1 == N2: the N1 table serves both)
  static constexpr int OFF_TAB = OFF_STWB + (N1 == N2 ? 0 : ((NSTWB * 8 + 127) / 128) * 128);
  // per stage: the pass-A tile's twiddle tables atab[32][WA], wtab[N1/32][WA]
  static constexpr int TABS = 32 * WA + (N1 / 32) * WA;
  static constexpr int OFF_BAR = OFF_TAB + 2 * TABS * 8;
  // barriers full[2] and empty[2], the fill log[8] and done counts[8], the
  // producer's and the reporter's fill counts
  static constexpr int SMEM = OFF_BAR + 192 + 1024;  // + alignment slack
  static_assert(N1 >= 256 && N1 <= 1024 && N2 >= 256 && N2 <= 1024, "tile shapes cover 256..1024");
};

// ------------------------------------------------------------ PTX helpers
__device__ __forceinline__ unsigned su32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(b)) : "memory");
}
// Raises the phase's expected transaction bytes without arriving.
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* b, unsigned bytes) {
  asm volatile("mbarrier.expect_tx.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(su32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase of parity `parity` to complete.
__device__ __forceinline__ bool mbar_wait(unsigned long long* b, unsigned parity, long long limit) {
  for (long long i = 0;; i++) {
    if (mbar_test(b, parity)) return true;
    if (i >= limit) return false;
    __nanosleep(64);
  }
}
// 2-D tile of the tensor map at (x, y) into shared memory, completing on bar.
__device__ __forceinline__ void tma_load_2d(void* dst, const TensorMap* map, int x, int y, unsigned long long* bar,
                                            unsigned long long pol) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1, {%2, %3}], [%4], %5;" ::"r"(su32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(su32(bar)), "l"(pol)
      : "memory");
}
// Contiguous bytes (multiple of 16, both addresses 16-byte aligned).
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, unsigned long long* bar,
                                          unsigned long long pol) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::
          "r"(su32(dst)),
      "l"(src), "r"(bytes), "r"(su32(bar)), "l"(pol)
      : "memory");
}
// Orders this thread's generic-proxy global accesses with async-proxy ones.
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }
__device__ __forceinline__ void consumers_sync() { asm volatile("bar.sync 1, %0;" ::"n"(kConsumers) : "memory"); }
// Barrier over the consumer warps that returns the OR of `pred`.
__device__ __forceinline__ bool consumers_sync_or(bool pred) {
  unsigned r;
  asm volatile(
      "{\n.reg .pred p, q;\nsetp.ne.u32 p, %1, 0;\nbar.red.or.pred q, 1, %2, p;\nselp.u32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"((unsigned)pred), "n"(kConsumers)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ unsigned long long policy_first() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ unsigned long long policy_last() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ unsigned long long policy_normal() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ void st_hint(float2* p, float2 v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(v.x), "f"(v.y), "l"(pol)
               : "memory");
}

// Records the first error of the launch (and in the plan's host word).
__device__ __forceinline__ void report(const PipeArgs& a, int code) {
  atomicCAS(a.err, 0, code);
  if (a.sticky) {
    *(volatile int*)a.sticky = code;
    __threadfence_system();
  }
}

// Task of ticket t: pass (A or B), transform k, tile index.
template <int TA, int TB>
__device__ __forceinline__ void decode(long long t, long long count, int lead, bool& is_a, long long& k,
                                       long long& tile) {
  const long long per = TA + TB, pairs = count - lead;
  if (t < lead * (long long)TA) {
    is_a = true;
    k = t / TA;
    tile = t - k * TA;
  } else if (t - lead * (long long)TA < pairs * per) {
    const long long u = t - lead * (long long)TA, j = u / per, r = u - j * per;
    is_a = r < TA;
    k = is_a ? j + lead : j;
    tile = is_a ? r : r - TA;
  } else {
    const long long v = t - lead * (long long)TA - pairs * per;
    is_a = false;
    k = pairs + v / TB;
    tile = v - (k - pairs) * TB;
  }
}

// ------------------------------------------------------------ producer
// Fill u of the launch (u = 0, 1, ...) goes to stage u % 2, its ticket to
// log[u % kLog]; the consumers and the reporter walk the fills in the same
// order. The producer refills a stage once its consumers are done with it
// (the `empty` barrier); the reporter follows behind, up to kLog fills, and
// publishes finished tiles to the other CTAs.
constexpr int kLog = 8;
struct Ctl {
  unsigned long long* full;   // [2]: the producer's arrival + the copies' bytes
  unsigned long long* empty;  // [2]: one arrival per consumer warp
  long long* log;             // [kLog]: ticket of each fill, -1 ends the launch
  int* done;                  // [kLog]: consumer warps done with the fill
  volatile int* filled;       // fills made (the log entry is written first)
  volatile int* reported;     // fills published by the reporter
};

// The producer: one thread takes tickets (one ahead, so the atomic's
// latency overlaps the current tile), waits for dependencies (a counter seen
// complete once is not polled again) and issues the copies. A pass-A tile's
// copy brings the tile's twiddle tables along (plan-time, FP64 rounded
// once):
//   atab[r][t] = w_N^(c R0 r),  wtab[j][t] = w_N^(c j),  c = c0 + t,
// so the consumers' inter-pass twiddle w_N^(c k1) (k1 = j + R0 r) is two
// shared loads and one product.
template <int N1, int N2>
__device__ __forceinline__ void producer(const TensorMap* tin, const PipeArgs& a, float2* stage, float2* tabs,
                                         const Ctl& c) {
  using S = Shape<N1, N2>;
  constexpr int W = S::WA;
  constexpr unsigned kTabBytes = S::TABS * 8;
  const long long total = a.count * (long long)(S::TA + S::TB);
  const unsigned long long pol_in = a.hints ? policy_first() : policy_normal();
  const unsigned long long pol_ring = a.hints ? policy_last() : policy_normal();
  const int* seen = nullptr;  // dependency counter last seen complete
  long long next = (long long)atomicAdd(a.ticket, 1ull);
  for (long long u = 0;; u++) {
    const int s = (int)(u & 1);
    // The stage's previous fill (u - 2) is consumed, and the log slot's
    // previous fill (u - kLog) is published.
    bool free_stage = u < 2 || mbar_wait(&c.empty[s], (unsigned)(((u - 2) >> 1) & 1), 16 * a.spin_limit);
    for (long long it = 0; free_stage && *c.reported < u - kLog + 1; it++) {
      if (it >= 16 * a.spin_limit) free_stage = false;
      __nanosleep(64);
    }
    bool end = !free_stage;
    if (!free_stage) report(a, 4);
    const long long t = next;
    if (!end) end = t >= total || *(volatile int*)a.err != 0;
    bool is_a = true;
    long long k = 0, tile = 0;
    if (!end) {
      next = (long long)atomicAdd(a.ticket, 1ull);  // used next iteration
      decode<S::TA, S::TB>(t, a.count, a.lead, is_a, k, tile);
      const int* w = is_a ? (k >= a.ring_slots ? a.done_b + (k - a.ring_slots) : nullptr) : a.done_a + k;
      const int need = (is_a ? S::TB : S::TA) + (!is_a && k == 0 && a.stall > 0 ? 1 : 0);
      if (w && w != seen) {
        for (long long it = 0; ld_acquire(w) < need; it++) {
          if (it >= a.spin_limit || *(volatile int*)a.err) {
            report(a, 3);
            end = true;
            break;
          }
          __nanosleep(256);
        }
        if (!end) seen = w;
      }
    }
    if (end) {
      // The end marker goes to the next stage when it is free; the
      // consumers and the reporter leave when they reach it. Copies already
      // issued are consumed before that.
      if (free_stage) {
        c.log[u % kLog] = -1;
        __threadfence_block();
        *c.filled = (int)(u + 1);
        mbar_arrive(&c.full[s]);
      }
      return;
    }
    float2* dst = stage + s * kTileElems;
    c.log[u % kLog] = t;
    __threadfence_block();
    *c.filled = (int)(u + 1);
    if (is_a) {
      mbar_expect_tx(&c.full[s], kTileElems * 8 + kTabBytes);
#pragma unroll
      for (int q = 0; q < N1 / S::BOXR; q++)
        tma_load_2d(dst + q * S::BOXR * W, tin, (int)tile * W, (int)(k * N1 + q * S::BOXR), &c.full[s], pol_in);
      bulk_load(tabs + s * S::TABS, a.tiles_tw + tile * S::TABS, kTabBytes, &c.full[s], pol_ring);
    } else {
      // The ring rows were written through the generic proxy by other CTAs
      // (release / acquire on done_a); the bulk copy reads them through the
      // async proxy.
      fence_proxy_async_global();
      mbar_expect_tx(&c.full[s], kTileElems * 8);
      const float2* src = a.ring + (k % a.ring_slots) * (long long)S::N + tile * (long long)S::WB * N2;
      bulk_load(dst, src, kTileElems * 8, &c.full[s], pol_ring);
    }
    // The phase's one arrival: releases the log entry to the consumers; the
    // phase completes when the copies' bytes have landed as well.
    mbar_arrive(&c.full[s]);
  }
}

// ------------------------------------------------------------ reporter
// Publishes finished tiles to the other CTAs. Each consumer warp that is
// done with fill u adds one to done[u % kLog] (release, CTA scope); when it
// reaches kConsumerWarps the reporter (acquire) has seen all of the tile's
// stores, and one acq_rel fence at GPU scope releases them before the
// tile's counter goes up (plus a proxy fence for ring rows, which bulk
// copies read next). The fence waits for those stores to reach L2
// (microseconds), so it runs here, off the producer's path, once for every
// tile that finished meanwhile.
template <int TA, int TB>
__device__ __forceinline__ void reporter(const PipeArgs& a, const Ctl& c) {
  const long long limit = 32 * a.spin_limit;
  long long u = 0;
  for (;;) {
    long long it = 0;
    while (*c.filled <= u) {
      if (++it > limit) return;
      __nanosleep(64);
    }
    __threadfence_block();
    if (c.log[u % kLog] < 0) return;
    // Every fill from u on whose consumers are done.
    long long v = u;
    bool any_a = false;
    for (it = 0;;) {
      if (v < *c.filled) {
        __threadfence_block();
        const long long t = c.log[v % kLog];
        int d;
        asm volatile("ld.acquire.cta.shared::cta.b32 %0, [%1];" : "=r"(d) : "r"(su32(c.done + v % kLog)) : "memory");
        if (t >= 0 && d == kConsumerWarps) {
          bool is_a;
          long long k, tile;
          decode<TA, TB>(t, a.count, a.lead, is_a, k, tile);
          any_a |= is_a;
          v++;
          continue;
        }
      }
      if (v > u) break;
      if (++it > limit) {
        report(a, 6);
        return;
      }
      __nanosleep(64);
    }
    if (any_a) fence_proxy_async_global();  // the ring rows are read next by bulk copies
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
    for (; u < v; u++) {
      bool is_a;
      long long k, tile;
      decode<TA, TB>(c.log[u % kLog], a.count, a.lead, is_a, k, tile);
      atomicAdd(is_a ? a.done_a + k : a.done_b + k, 1);
      c.done[u % kLog] = 0;
    }
    __threadfence_block();
    *c.reported = (int)u;
  }
}

// ------------------------------------------------------------ consumer tiles
// A consumer warp has read everything it needs from the stage (the data in
// the first pass, the tile's twiddles into registers): it frees the stage,
// so the producer's copy of the tile after next overlaps the second pass.
__device__ __forceinline__ void release_stage(unsigned long long* empty) {
  __syncwarp();  // every lane's reads come before lane 0's arrival
  if ((threadIdx.x & 31) == 0) mbar_arrive(empty);
}

// Pass A tile: columns c0 .. c0 + WA - 1 of transform k. The stage holds the
// tile as [n1][t] (TMA box rows); the first pass is N1/32-point butterflies
// (K0 per thread) over n1 with stride 32, the second radix 32 with stage
// twiddles w_N1^(j r); the result row k1 = j + (N1/32) r goes to the ring
// times scale w_N^(k1 c) (the tile's tables, copied with its data). The
// stage is released after the first pass.
template <int N1, int N2, bool BACK>
__device__ __forceinline__ void tile_a(const PipeArgs& a, const float2* stg, float2* xch, const float2* stw,
                                       const float2* atab, long long k, int c0, int tid, unsigned long long* empty,
                                       unsigned long long pol_ring) {
  using S = Shape<N1, N2>;
  constexpr int W = S::WA, R0 = N1 / 32, K0 = 32 / R0, LD = S::LDA;
  const float2* wtab = atab + 32 * W;
  {
    float2 v[K0][R0];
#pragma unroll
    for (int kk = 0; kk < K0; kk++) {
      const int bf = tid + kk * kConsumers, t = bf % W, j = bf / W;
#pragma unroll
      for (int r = 0; r < R0; r++) {
        const float2 x = stg[(j + 32 * r) * W + t];
        v[kk][r] = BACK ? cconj(x) : x;
      }
    }
#pragma unroll
    for (int kk = 0; kk < K0; kk++) {
      const int bf = tid + kk * kConsumers, t = bf % W, j = bf / W;
      Dft<R0>::run(v[kk]);
#pragma unroll
      for (int r = 0; r < R0; r++) xch[t * LD + xch_pad(j * R0 + r)] = v[kk][r];
    }
  }
  // This thread's inter-pass twiddles scale w_N^(c (j + R0 r)), read now so
  // the stage (data and tables) is free before the second pass.
  const int t = tid % W, j = tid / W;
  float2 tw[32];
  {
    const float2 wj = cscale(wtab[j * W + t], a.scale);
#pragma unroll
    for (int r = 0; r < 32; r++) tw[r] = cmul(wj, atab[r * W + t]);
  }
  release_stage(empty);
  consumers_sync();
  float2 u[32];
#pragma unroll
  for (int r = 0; r < 32; r++) u[r] = xch[t * LD + xch_pad(j + R0 * r)];
#pragma unroll
  for (int r = 1; r < 32; r++) u[r] = cmul(u[r], stw[(r - 1) * R0 + j]);
  Dft<32>::run(u);
  float2* dst = a.ring + (k % a.ring_slots) * (long long)S::N + c0 + t;
#pragma unroll
  for (int r = 0; r < 32; r++) st_hint(dst + (long long)(j + R0 * r) * N2, cmul(u[r], tw[r]), pol_ring);
}

// Pass B tile: rows r0 .. r0 + WB - 1 of transform k's intermediate, held
// [t][n2] in the stage. First pass with threads along each row (contiguous
// reads), second radix 32 with threads across rows so the transposed store
// X[r0 + t + N1 k2] is contiguous over t.
template <int N1, int N2, bool BACK>
__device__ __forceinline__ void tile_b(const PipeArgs& a, const float2* stg, float2* xch, const float2* stw,
                                       long long k, int r0, int tid, unsigned long long* empty,
                                       unsigned long long pol_out) {
  using S = Shape<N1, N2>;
  constexpr int W = S::WB, R0 = N2 / 32, K0 = 32 / R0, LD = S::LDB;
  {
    float2 v[K0][R0];
#pragma unroll
    for (int kk = 0; kk < K0; kk++) {
      const int bf = tid + kk * kConsumers, t = bf / 32, j = bf % 32;
#pragma unroll
      for (int r = 0; r < R0; r++) v[kk][r] = stg[t * N2 + j + 32 * r];
    }
#pragma unroll
    for (int kk = 0; kk < K0; kk++) {
      const int bf = tid + kk * kConsumers, t = bf / 32, j = bf % 32;
      Dft<R0>::run(v[kk]);
#pragma unroll
      for (int r = 0; r < R0; r++) xch[t * LD + xch_pad(j * R0 + r)] = v[kk][r];
    }
  }
  release_stage(empty);
  consumers_sync();
  const int t = tid % W, j = tid / W;
  float2 u[32];
#pragma unroll
  for (int r = 0; r < 32; r++) u[r] = xch[t * LD + xch_pad(j + R0 * r)];
#pragma unroll
  for (int r = 1; r < 32; r++) u[r] = cmul(u[r], stw[(r - 1) * R0 + j]);
  Dft<32>::run(u);
  float2* dst = a.out + k * (long long)S::N + r0 + t;
#pragma unroll
  for (int r = 0; r < 32; r++) st_hint(dst + (long long)(j + R0 * r) * N1, BACK ? cconj(u[r]) : u[r], pol_out);
}

// A consumer warp is done with a tile: it counts itself done for the
// reporter (release: its stores come first).
__device__ __forceinline__ void finish_tile(int* done) {
  __syncwarp();  // orders every lane's stores before lane 0's release
  if ((threadIdx.x & 31) == 0)
    asm volatile("red.release.cta.shared::cta.add.s32 [%0], 1;" ::"r"(su32(done)) : "memory");
}

template <int N1, int N2, bool BACK>
__global__ void __launch_bounds__(kThreads, 1) k_pipe(const __grid_constant__ TensorMap tin, const PipeArgs a) {
  using S = Shape<N1, N2>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* base = smem_raw + ((1024 - (su32(smem_raw) & 1023)) & 1023);
  float2* stage = reinterpret_cast<float2*>(base);
  float2* xch = reinterpret_cast<float2*>(base + S::OFF_XCH);
  float2* stwa = reinterpret_cast<float2*>(base + S::OFF_STWA);
  float2* stwb = reinterpret_cast<float2*>(base + S::OFF_STWB);
  float2* tabs = reinterpret_cast<float2*>(base + S::OFF_TAB);
  Ctl c;
  c.full = reinterpret_cast<unsigned long long*>(base + S::OFF_BAR);
  c.empty = c.full + 2;
  c.log = reinterpret_cast<long long*>(c.full + 4);
  c.done = reinterpret_cast<int*>(c.log + kLog);
  c.filled = c.done + kLog;
  c.reported = c.filled + 1;
  const int tid = threadIdx.x;
  // Radix-32 stage twiddles (the second pass's block of the stage tables).
  for (int i = tid; i < S::NSTWA; i += kThreads) stwa[i] = a.stw_a[N1 / 32 - 1 + i];
  if (N1 != N2)
    for (int i = tid; i < S::NSTWB; i += kThreads) stwb[i] = a.stw_b[N2 / 32 - 1 + i];
  if (tid == 0) {
    // full: the producer's one arrival per fill plus the copies' bytes;
    // empty: one arrival per consumer warp when it is done with the tile.
    mbar_init(&c.full[0], 1);
    mbar_init(&c.full[1], 1);
    mbar_init(&c.empty[0], kConsumerWarps);
    mbar_init(&c.empty[1], kConsumerWarps);
    for (int q = 0; q < kLog; q++) c.done[q] = 0;
    *c.filled = 0;
    *c.reported = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid >= kConsumers) {
    if (tid == kConsumers) producer<N1, N2>(&tin, a, stage, tabs, c);
    if (tid == kConsumers + 32) reporter<S::TA, S::TB>(a, c);
    return;
  }
  const unsigned long long pol_ring = a.hints ? policy_last() : policy_normal();
  const unsigned long long pol_out = a.hints ? policy_first() : policy_normal();
  for (long long u = 0;; u++) {
    const int s = (int)(u & 1);
    // Longer than the producer's waits, so a producer that gives up reaches
    // the consumers with its end marker first.
    const bool ok = mbar_wait(&c.full[s], (unsigned)((u >> 1) & 1), 16 * a.spin_limit);
    // One barrier per tile boundary: every consumer has finished the
    // previous tile (the exchange buffer is free), and all agree whether to
    // leave.
    const bool abort = consumers_sync_or(!ok);
    if (abort) {
      if (tid == 0) report(a, 5);
      return;
    }
    const long long t = c.log[u % kLog];
    if (t < 0) return;
    bool is_a;
    long long k, tile;
    decode<S::TA, S::TB>(t, a.count, a.lead, is_a, k, tile);
    const float2* stg = stage + s * kTileElems;
    if (is_a)
      tile_a<N1, N2, BACK>(a, stg, xch, stwa, tabs + s * S::TABS, k, (int)tile * S::WA, tid, &c.empty[s], pol_ring);
    else
      tile_b<N1, N2, BACK>(a, stg, xch, N1 == N2 ? stwa : stwb, k, (int)tile * S::WB, tid, &c.empty[s], pol_out);
    finish_tile(c.done + u % kLog);
  }
}

}  // namespace pipe
}  // namespace chfft
