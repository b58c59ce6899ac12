// Tensor-core core policy: the radix-16 passes of a length-N FFT run as
// small complex matrix products on the fifth-generation tensor cores.
//
// A radix-16 Stockham pass over R butterflies is the real product
//   D (R x 32) = A (R x 32) * B^T,  B (32 x 32) = [[C, S], [-S, C]]
// where row r of A holds the 16 twiddled inputs of butterfly r (16 real
// parts, then 16 imaginary parts), C_jk = cos(2 pi jk / 16), S_jk =
// sin(2 pi jk / 16), and row r of D holds its 16 outputs the same way.
// FP32 operands are split into 16-bit parts, x = hi + lo (+ mid), each row
// scaled by a power of two so its largest entry is below 2^14 (no FP16
// overflow, small parts stay normal), and the products accumulate in FP32
// in tensor memory:
//   PREC 1: FP16 hi + lo, products hi*hi + lo*hi + hi*lo   (3 MMAs per K step)
//   PREC 2: BF16 hi + lo, the same three products
//   PREC 3: BF16 hi + mid + lo, the six products above 2^-24 (6 MMAs)
// A first pass of radix R0 in {1, 2, 4, 8} (N = R0 * 16^S16) runs on the FP32
// cores. The data tile, the Stockham order and the stage twiddle table are
// those of the FP32 engine (engine.cuh), so this policy drops into the same
// kernels (rows, four-step columns, transposing rows).
//
// One CTA of kTcThreads threads; the M = 128 row tiles of a pass are spread
// over warp quarters (a warp reads tensor-memory lanes 32 * (warp % 4)..+31).
// Waits on the MMA completion barrier are bounded: on time-out the CTA
// records an error in the core's error word, waits (bounded) once more,
// frees its tensor memory and returns.
#pragma once

#include "engine.cuh"
#include "tc.cuh"

namespace chfft {

namespace tcd {

__device__ __forceinline__ unsigned pack_f16x2(float lo_elem, float hi_elem) {
  unsigned r;
  asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi_elem), "f"(lo_elem));
  return r;
}
__device__ __forceinline__ void unpack_f16x2(unsigned v, float& a, float& b) {
  asm("{\n.reg .b16 l, h;\nmov.b32 {l, h}, %2;\ncvt.f32.f16 %0, l;\ncvt.f32.f16 %1, h;\n}\n"
      : "=f"(a), "=f"(b)
      : "r"(v));
}
__device__ __forceinline__ unsigned pack_bf16x2(float lo_elem, float hi_elem) {
  unsigned r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi_elem), "f"(lo_elem));
  return r;
}
__device__ __forceinline__ void unpack_bf16x2(unsigned v, float& a, float& b) {
  a = __uint_as_float(v << 16);
  b = __uint_as_float(v & 0xFFFF0000u);
}

// Splits the pair (x0, x1) into NPART packed 16-bit parts, largest first.
template <int PREC>
__device__ __forceinline__ void split_pair(float x0, float x1, unsigned* parts) {
  constexpr int NP = PREC == 3 ? 3 : 2;
#pragma unroll
  for (int q = 0; q < NP; q++) {
    float a, b;
    if (PREC == 1) {
      parts[q] = pack_f16x2(x0, x1);
      unpack_f16x2(parts[q], a, b);
    } else {
      parts[q] = pack_bf16x2(x0, x1);
      unpack_bf16x2(parts[q], a, b);
    }
    x0 -= a;
    x1 -= b;
  }
}

// 2^k as a float for |k| < 126.
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((127 + k) << 23); }

// cos / sin of 2 pi m / 16, evaluated in double at compile time, rounded once.
struct Dft16 {
  float c[16], s[16];
};
__host__ __device__ constexpr Dft16 make_dft16() {
  Dft16 t{};
  for (int m = 0; m < 16; m++) {
    t.c[m] = (float)ct::cos2pi(m, 16);
    t.s[m] = (float)ct::sin2pi(m, 16);
  }
  return t;
}
__device__ constexpr Dft16 kDft16 = make_dft16();

}  // namespace tcd

// TMINOR: thread mapping of the load / store phases (column tiles);
// N: FFT length; TPB: sequences per CTA; LD: tile stride (pad period 16);
// PREC: 1 FP16x2, 2 BF16x2, 3 BF16x3; R0: first (FP32) radix; S16: number
// of tensor-core radix-16 passes.
template <bool TMINOR, int N, int TPB, int LD, int PREC, int R0, int S16>
struct TcCore {
  static constexpr bool kK1 = false;
  static constexpr bool kStatic = true;
  static constexpr int kThreads = kTcThreads;
  static constexpr int P = 16;                       // tile pad period
  static constexpr int NP = PREC == 3 ? 3 : 2;       // 16-bit parts per operand
  static constexpr int ROWS = TPB * (N / 16);        // butterflies per radix-16 pass
  static constexpr int T = ROWS / 128;               // M = 128 row tiles
  static constexpr int NPROD = PREC == 3 ? 6 : 3;
  static constexpr int TILE_BYTES = TPB * LD * 8;    // f32 complex data tile
  static constexpr int A_OFF = (TILE_BYTES + 1023) / 1024 * 1024;
  static constexpr int A_BYTES = T * NP * 128 * 64;  // row tiles x parts x 128 rows x 64 bytes
  static constexpr int B_OFF = A_OFF + A_BYTES;
  static constexpr int B_BYTES = NP * 32 * 64;
  static constexpr int BAR_OFF = B_OFF + B_BYTES;
  static constexpr int SMEM = BAR_OFF + 16;
  // Launch bounds: as many resident CTAs as the shared memory allows, up to
  // three (79 registers at three: no spills).
  static constexpr int kMinBlocks = 3 * SMEM <= 227 * 1024 ? 3 : 2 * SMEM <= 227 * 1024 ? 2 : 1;
  static constexpr int TMEM_COLS = (32 * T <= 32) ? 32 : (32 * T <= 64) ? 64 : (32 * T <= 128) ? 128 : (32 * T <= 256) ? 256 : 512;
  static_assert(N == R0 * (S16 == 1 ? 16 : S16 == 2 ? 256 : S16 == 3 ? 4096 : 65536), "N = R0 * 16^S16");
  static_assert(ROWS % 128 == 0 && T >= 1 && T <= 16, "radix-16 rows must fill M = 128 tiles");
  static_assert(R0 == 1 || R0 == 2 || R0 == 4 || R0 == 8, "first radix");
  static_assert(LD >= N + N / 16, "tile stride");

  template <typename C>
  __device__ __forceinline__ static SmemIO<C, P> tile(unsigned char* base, int) {
    return SmemIO<C, P>{reinterpret_cast<C*>(base), LD};
  }

  // Row-major parts -> canonical K-major layout, one thread per row.
  __device__ __forceinline__ static void stage_row(unsigned char* sa, int row, const float (&re)[16],
                                                   const float (&im)[16]) {
    const int t = row >> 7, r = row & 127;
#pragma unroll
    for (int kb = 0; kb < 4; kb++) {
      unsigned w[NP][4];
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const int k = kb * 8 + 2 * e;
        const float x0 = k < 16 ? re[k] : im[k - 16];
        const float x1 = k < 16 ? re[k + 1] : im[k - 15];
        unsigned parts[NP];
        tcd::split_pair<PREC>(x0, x1, parts);
#pragma unroll
        for (int q = 0; q < NP; q++) w[q][e] = parts[q];
      }
#pragma unroll
      for (int q = 0; q < NP; q++) {
        unsigned char* dst = sa + (t * NP + q) * (128 * 64) + tc::kmajor_offset(r, kb * 8, 32);
        *reinterpret_cast<uint4*>(dst) = make_uint4(w[q][0], w[q][1], w[q][2], w[q][3]);
      }
    }
  }

  // The DFT-16 matrix B (32 x 32, row n' = output component, K = input
  // component) in NP parts, from FP64 values rounded once.
  __device__ __forceinline__ static void build_b(unsigned char* sb) {
    for (int i = threadIdx.x; i < 32 * 16; i += blockDim.x) {
      const int n = i / 16, kp = i % 16;  // kp: pair of K entries (2 kp, 2 kp + 1)
      float v[2];
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int k = 2 * kp + h;
        const int j = n & 15, kk = k & 15;
        const float c = tcd::kDft16.c[(j * kk) & 15], s = tcd::kDft16.s[(j * kk) & 15];
        const bool re_out = n < 16, re_in = k < 16;
        // Re Y = C a + S b; Im Y = -S a + C b (forward, w = exp(-2 pi i / 16)).
        v[h] = (float)(re_out ? (re_in ? c : s) : (re_in ? -s : c));
      }
      unsigned parts[NP];
      tcd::split_pair<PREC>(v[0], v[1], parts);
#pragma unroll
      for (int q = 0; q < NP; q++)
        *reinterpret_cast<unsigned*>(sb + q * (32 * 64) + tc::kmajor_offset(n, 2 * kp, 32)) = parts[q];
    }
  }

  template <bool ROWS_FIRST = false, typename C, class Ld, class St>
  __device__ __forceinline__ static void run(const CoreDesc& d, int, const SmemIO<C, P>& sm, const Ld& ld,
                                             const St& st) {
    static_assert(same_type<C, float2>::value, "tensor-core passes run on f32 data");
    unsigned char* base = reinterpret_cast<unsigned char*>(sm.s);
    unsigned char* sa = base + A_OFF;
    unsigned char* sb = base + B_OFF;
    unsigned long long* mbar = reinterpret_cast<unsigned long long*>(base + BAR_OFF);
    unsigned* slot = reinterpret_cast<unsigned*>(base + BAR_OFF + 8);
    int* timed_out = reinterpret_cast<int*>(base + BAR_OFF + 12);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const C* stw = static_cast<const C*>(d.stw);

    if (warp == 0) tc::tmem_alloc(slot, TMEM_COLS);
    if (tid == 0) {
      tc::mbar_init(mbar, 1);
      *timed_out = 0;
    }
    build_b(sb);
    load_phase<ROWS_FIRST ? false : TMINOR>(sm, N, TPB, ld);  // ends with a barrier
    int Ns = 1, off = 0;
    if constexpr (R0 > 1) {
      constexpr int EPT = R0 * ((TPB * (N / R0) + kTcThreads - 1) / kTcThreads);
      pass_body<R0, false, false, true, EPT>(N, 1, TPB, stw, sm, sm);
      Ns = R0;
      off = R0 - 1;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const unsigned tmem = *slot;
    constexpr int NB = N / 16;
    constexpr int ROW_ITERS = (ROWS + kTcThreads - 1) / kTcThreads;  // row slots per thread
    bool ok = true;
    for (int s = 0; s < S16; s++) {
      // Rows of this thread: row = 128 t + 32 (warp % 4) + lane, t = warp / 4 + k * (warps / 4).
      int scale_e[ROW_ITERS];
#pragma unroll
      for (int it = 0; it < ROW_ITERS; it++) {
        const int t = (warp >> 2) + it * (kTcThreads / 128);
        const int row = 128 * t + 32 * (warp & 3) + lane;
        scale_e[it] = 0;
        if (t >= T) continue;
        const int seq = row / NB, j = row - seq * NB;
        const int jm = j % Ns;
        float re[16], im[16], mx = 0.f;
#pragma unroll
        for (int r = 0; r < 16; r++) {
          C v = sm.load(seq, j + r * NB);
          if (r > 0 && Ns > 1) v = cmul(v, __ldg(&stw[off + (r - 1) * Ns + jm]));
          re[r] = v.x;
          im[r] = v.y;
          mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
        }
        int e = 0;
        if (mx > 0.f) {
          frexpf(mx, &e);  // mx < 2^e
          e = max(-100, min(100, e));
        }
        scale_e[it] = e;
        const float sc = tcd::pow2f(14 - e);
#pragma unroll
        for (int r = 0; r < 16; r++) {
          re[r] *= sc;
          im[r] *= sc;
        }
        stage_row(sa, row, re, im);
      }
      tc::fence_async_smem();
      tc::fence_before_sync();
      __syncthreads();
      tc::fence_after_sync();
      if (tid == 0) {
        constexpr unsigned id = tc::idesc_f16(128, 32, PREC != 1);
        const unsigned a0 = tc::smem_u32(sa), b0 = tc::smem_u32(sb);
        // Products (A part, B part) above the 2^-24 level, largest first.
        constexpr int pa[6] = {0, 1, 0, 1, 0, 2};
        constexpr int pb[6] = {0, 0, 1, 1, 2, 0};
        for (int t = 0; t < T; t++) {
          int acc = 0;
          for (int p = 0; p < NPROD; p++) {
            const int qa = PREC == 3 ? pa[p] : (p == 0 ? 0 : p == 1 ? 1 : 0);
            const int qb = PREC == 3 ? pb[p] : (p == 2 ? 1 : 0);
            for (int ks = 0; ks < 2; ks++) {
              const unsigned long long da = tc::smem_desc(a0 + (t * NP + qa) * (128 * 64) + ks * 256, 128, 512);
              const unsigned long long db = tc::smem_desc(b0 + qb * (32 * 64) + ks * 256, 128, 512);
              tc::mma_f16(tmem + 32 * t, da, db, id, acc);
              acc = 1;
            }
          }
        }
        tc::commit(mbar);
      }
      if (!tc::mbar_wait(mbar, s & 1, 1 << 22)) atomicExch(timed_out, 1);
      tc::fence_after_sync();
      __syncthreads();
      if (*timed_out) {  // uniform across the CTA
        if (d.err && tid == 0) atomicExch(d.err, 2);
        tc::mbar_wait(mbar, s & 1, 1 << 22);
        ok = false;
        break;
      }
#pragma unroll
      for (int it = 0; it < ROW_ITERS; it++) {
        const int t = (warp >> 2) + it * (kTcThreads / 128);
        if (t >= T) continue;
        const int row = 128 * t + 32 * (warp & 3) + lane;
        float y[32];
        tc::tmem_ld_32x32(tmem + ((unsigned)(32 * (warp & 3)) << 16) + 32 * t, y);
        const int seq = row / NB, j = row - seq * NB;
        const int jm = j % Ns;
        const int bse = (j - jm) * 16 + jm;
        const float us = tcd::pow2f(scale_e[it] - 14);
#pragma unroll
        for (int r = 0; r < 16; r++) sm.store(seq, bse + r * Ns, mk(y[r] * us, y[16 + r] * us));
      }
      off += 15 * Ns;
      Ns *= 16;
      tc::fence_before_sync();
      __syncthreads();
      tc::fence_after_sync();
    }
    if (ok) store_phase<TMINOR>(sm, N, TPB, st);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, TMEM_COLS);
  }
};

}  // namespace chfft
