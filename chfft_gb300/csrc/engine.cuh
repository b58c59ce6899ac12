// Block-level Stockham FFT engine.
//
// A CTA transforms `tpb` independent sequences of length n held in shared
// memory. Each radix-R pass reads R elements with stride n/R, applies the
// stage twiddles, runs the register butterfly and writes them back in
// self-sorting (Stockham) order, so no digit-reversal permutation is ever
// materialised — the GPU counterpart of chfft's gather list + in-order DIT
// stages (src/mixed_radix.rs:24-166, src/precompute_utils.rs:70-91).
//
// Pass order. A Stockham FFT is correct for any order of its radices, so the
// shared-memory passes run in a canonical order (16, 8, 4, 2, 10, 5, 3, 7),
// one loop per radix. Each radix body then appears once in straight-line
// code, which keeps every pass in registers (a runtime switch over radices
// inside one pass loop makes the compiler keep the butterfly arrays in local
// memory). Hot kernels fuse their global load into the first pass and their
// store into the last pass (a switch on the radix outside any loop); the
// others use a load phase and a store phase around the shared-memory passes.
//
// Thread mapping: butterfly b in [0, tpb*n/R). TMINOR=false gives
// (t = b / nb, j = b % nb): consecutive threads walk one sequence, which
// coalesces contiguous rows. TMINOR=true gives (t = b % tpb, j = b / tpb):
// consecutive threads walk adjacent sequences, which coalesces column tiles.
#pragma once

#include "common.cuh"

namespace chfft {

constexpr int kMaxThreads = 512;  // threads per CTA, every kernel
constexpr int kTcThreads = 256;   // threads per CTA of the tensor-core core (tc_core.cuh)
constexpr int kNumRadix = 9;
// Canonical radix order of the shared-memory passes. Radix 32 (last) only
// appears in the stage lists of compile-time-stage kernels with 32 elements
// per thread (f32): the run-time-stage loops below cover the first eight.
CHFFT_HD constexpr int radix_at(int i) {
  return i == 0 ? 16 : i == 1 ? 8 : i == 2 ? 4 : i == 3 ? 2 : i == 4 ? 10 : i == 5 ? 5 : i == 6 ? 3 : i == 7 ? 7 : 32;
}

// Complex elements one thread holds during a pass: 32 (64 registers) for
// f32, 16 (64 registers) for f64. A pass of radix R gives each thread up to
// EPT/R butterflies. The K1 variants give every thread exactly one
// butterfly per pass (R elements): smaller code, fewer registers and more
// resident warps, usable when no pass has more than kMaxThreads butterflies
// per CTA.
template <typename C> struct Ept;
template <> struct Ept<float2> { static constexpr int value = 32; };
template <> struct Ept<double2> { static constexpr int value = 16; };

// Stage plan of one FFT length. The fused variants run rf, the `mid` passes
// in canonical order, then rl; the phased variants run the `all` passes in
// canonical order. Both orders compute the same transform.
struct StageList {
  int n;                 // FFT length
  int npass;             // total number of passes (0 for n == 1)
  int rf, rl;            // first / last radix of the fused order (npass >= 2)
  int mid[kNumRadix];    // fused order: pass counts between rf and rl
  int all[kNumRadix];    // phased order: pass counts
};

// Shared-memory placement of element i of sequence t: one pad slot per P
// elements (none for P = 0). The first pass stores with stride R (its
// radix); P = R makes that stride R+1, which is odd for even R and so
// conflict-free. The library kernels use P = 16.
template <int P>
CHFFT_HD int smem_index(int t, int i, int ld) {
  return t * ld + i + (P > 0 ? i / (P > 0 ? P : 1) : 0);
}
// Odd stride: adjacent sequences then start in different banks, which keeps
// the TMINOR (column tile) accesses conflict-free.
CHFFT_HD int smem_ld(int n, int p = 16) { return (n + (p > 0 ? n / p : 0)) | 1; }

template <typename C, int P = 16>
struct SmemIO {
  C* s;
  int ld;
  __device__ __forceinline__ C load(int t, int i) const { return s[smem_index<P>(t, i, ld)]; }
  __device__ __forceinline__ void store(int t, int i, C v) const { s[smem_index<P>(t, i, ld)] = v; }
};

template <class X> struct is_tile { static constexpr bool value = false; };
template <typename C, int P> struct is_tile<SmemIO<C, P>> { static constexpr bool value = true; };

template <bool TMINOR>
__device__ __forceinline__ void split_index(int b, int tpb, int nb, int& t, int& j) {
  if (TMINOR) {
    t = b % tpb;
    j = b / tpb;
  } else {
    t = b / nb;
    j = b - t * nb;
  }
}

// One radix-R Stockham pass: ld -> registers -> butterflies -> st. Ns is the
// product of the radices of the passes already run. All loads of the pass
// complete (barrier) before any store, so ld and st may be the same tile.
// Twiddles: tw is omega_n (entry r * (j mod Ns) * n / (Ns R)), or with STW
// this pass's block of the stage table, entry (r - 1) * Ns + (j mod Ns), so
// the r-th twiddles of a warp are one contiguous segment.
// EPT > 0 overrides the per-thread element budget of the non-K1 variant.
template <int R, bool TMINOR, bool K1, bool STW = false, int EPT = 0, typename C, class Ld, class St>
__device__ __forceinline__ void pass_body(int n, int Ns, int tpb, const C* __restrict__ tw, const Ld& ld,
                                          const St& st) {
  constexpr int K = K1 ? 1 : (EPT > 0 ? EPT : Ept<C>::value) / R;
  static_assert(K >= 1, "radix larger than the per-thread element budget");
  const int nb = n / R;
  const int total = tpb * nb;
  const int tw_step = (Ns > 1) ? n / (Ns * R) : 0;
  C v[K][R];
  int tt[K], jj[K];
#pragma unroll
  for (int k = 0; k < K; k++) {
    const int b = threadIdx.x + k * blockDim.x;
    jj[k] = -1;
    tt[k] = 0;
    if (b < total) {
      int t, j;
      split_index<TMINOR>(b, tpb, nb, t, j);
      tt[k] = t;
      jj[k] = j;
#pragma unroll
      for (int r = 0; r < R; r++) v[k][r] = ld.load(t, j + r * nb);
      if (Ns > 1) {
        if constexpr (STW) {
          const int jm = j % Ns;
#pragma unroll
          for (int r = 1; r < R; r++) v[k][r] = cmul(v[k][r], __ldg(&tw[(r - 1) * Ns + jm]));
        } else {
          const int step = (j % Ns) * tw_step;
#pragma unroll
          for (int r = 1; r < R; r++) v[k][r] = cmul(v[k][r], __ldg(&tw[r * step]));
        }
      }
      Dft<R>::run(v[k]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; k++) {
    if (jj[k] >= 0) {
      const int j = jj[k];
      const int jm = j % Ns;
      const int base = (j - jm) * R + jm;
#pragma unroll
      for (int r = 0; r < R; r++) st.store(tt[k], base + r * Ns, v[k][r]);
    }
  }
  __syncthreads();
}

// A single pass of runtime radix R (only ever called outside loops).
template <bool TMINOR, bool K1, typename C, class Ld, class St>
__device__ __forceinline__ void pass_any(int R, int n, int Ns, int tpb, const C* tw, const Ld& ld, const St& st) {
  switch (R) {
    case 16: pass_body<16, TMINOR, K1>(n,Ns, tpb, tw, ld, st); break;
    case 8: pass_body<8, TMINOR, K1>(n,Ns, tpb, tw, ld, st); break;
    case 4: pass_body<4, TMINOR, K1>(n,Ns, tpb, tw, ld, st); break;
    case 2: pass_body<2, TMINOR, K1>(n,Ns, tpb, tw, ld, st); break;
    case 10: pass_body<10, TMINOR, K1>(n,Ns, tpb, tw, ld, st); break;
    case 5: pass_body<5, TMINOR, K1>(n,Ns, tpb, tw, ld, st); break;
    case 3: pass_body<3, TMINOR, K1>(n,Ns, tpb, tw, ld, st); break;
    case 7: pass_body<7, TMINOR, K1>(n,Ns, tpb, tw, ld, st); break;
    default: break;
  }
}

// cnt[i] passes of radix radix_at(i) on the tile, in canonical order.
// Returns the updated radix product Ns.
template <bool TMINOR, bool K1, int EPT = 0, typename C>
__device__ __forceinline__ int smem_passes(const int* cnt, int n, int Ns, int tpb, const C* tw, const SmemIO<C>& sm) {
  for (int c = 0; c < cnt[0]; c++, Ns *= 16) pass_body<16, TMINOR, K1, false, EPT>(n, Ns, tpb, tw, sm, sm);
  for (int c = 0; c < cnt[1]; c++, Ns *= 8) pass_body<8, TMINOR, K1, false, EPT>(n, Ns, tpb, tw, sm, sm);
  for (int c = 0; c < cnt[2]; c++, Ns *= 4) pass_body<4, TMINOR, K1, false, EPT>(n, Ns, tpb, tw, sm, sm);
  for (int c = 0; c < cnt[3]; c++, Ns *= 2) pass_body<2, TMINOR, K1, false, EPT>(n, Ns, tpb, tw, sm, sm);
  for (int c = 0; c < cnt[4]; c++, Ns *= 10) pass_body<10, TMINOR, K1, false, EPT>(n, Ns, tpb, tw, sm, sm);
  for (int c = 0; c < cnt[5]; c++, Ns *= 5) pass_body<5, TMINOR, K1, false, EPT>(n, Ns, tpb, tw, sm, sm);
  for (int c = 0; c < cnt[6]; c++, Ns *= 3) pass_body<3, TMINOR, K1, false, EPT>(n, Ns, tpb, tw, sm, sm);
  for (int c = 0; c < cnt[7]; c++, Ns *= 7) pass_body<7, TMINOR, K1, false, EPT>(n, Ns, tpb, tw, sm, sm);
  return Ns;
}

// Element-wise phases between global memory and the tile.
template <bool TMINOR, typename C, class Ld>
__device__ __forceinline__ void load_phase(const SmemIO<C>& sm, int n, int tpb, const Ld& ld) {
  for (int b = threadIdx.x; b < tpb * n; b += blockDim.x) {
    int t, i;
    split_index<TMINOR>(b, tpb, n, t, i);
    sm.store(t, i, ld.load(t, i));
  }
  __syncthreads();
}

template <bool TMINOR, typename C, class St>
__device__ __forceinline__ void store_phase(const SmemIO<C>& sm, int n, int tpb, const St& st) {
  for (int b = threadIdx.x; b < tpb * n; b += blockDim.x) {
    int t, i;
    split_index<TMINOR>(b, tpb, n, t, i);
    st.store(t, i, sm.load(t, i));
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Bluestein (Chirp-Z) core for a length n that is not 7-smooth
// (src/chirpz.rs:87-203):
//   X_k = c_k * sum_j (x_j c_j) conj(c_{k-j}),  c_j = exp(-pi i (j^2 mod 2n)/n)
// evaluated as a length-M circular convolution, M >= 2n-1 and 7-smooth:
// FFT_M(x c) -> x B^ (B^ = FFT_M(conj c) / M) -> FFT_M^-1 -> x c_k. The chirp
// multiply and zero padding wrap the caller's loader, the inverse FFT runs as
// a conjugated forward FFT on the same shared-memory tile, and the output
// chirp wraps the caller's storer.
template <typename C, class Ld>
struct ChirpIn {
  const Ld& inner;
  const C* chirp;
  int n;
  __device__ __forceinline__ C load(int t, int i) const {
    using R = typename Real<C>::type;
    if (i >= n) return mk(R(0), R(0));
    return cmul(inner.load(t, i), __ldg(&chirp[i]));
  }
};

template <typename C, class St>
struct ChirpOut {
  const St& inner;
  const C* chirp;
  int n;
  __device__ __forceinline__ void store(int t, int i, C v) const {
    if (i < n) inner.store(t, i, cmul(cconj(v), __ldg(&chirp[i])));
  }
};

struct CoreDesc {
  StageList st;       // stages of the FFT actually run (length M for Bluestein)
  const void* tw;     // omega_{st.n} table
  int n;              // logical core length
  const void* chirp;  // Bluestein: c_j, j < n
  const void* bhat;   // Bluestein: FFT_M(conj c) / M
  const void* stw;    // stage twiddles of the fused pass order (compile-time-stage kernels)
  int* err;           // device error word (tensor-core cores: 2 = an MMA wait timed out), may be null
};

// Y <- conj(Y * B^) on every sequence of the tile.
template <bool TMINOR, typename C>
__device__ __forceinline__ void spectrum_phase(const SmemIO<C>& sm, int m, int tpb, const C* bhat) {
  for (int b = threadIdx.x; b < tpb * m; b += blockDim.x) {
    int t, i;
    split_index<TMINOR>(b, tpb, m, t, i);
    sm.store(t, i, cconj(cmul(sm.load(t, i), __ldg(&bhat[i]))));
  }
  __syncthreads();
}

// Core complex FFT of length d.n on the block's sequences: a mixed-radix
// Stockham FFT, or (BLUE) the fused Bluestein convolution. The storer is
// called for indices < d.n only. FUSED inlines the loader into the first
// pass and the storer into the last (when the stage list has >= 2 passes);
// otherwise they run as phases, and a loader or storer that is the tile
// itself runs no phase.
template <bool BLUE, bool TMINOR, bool FUSED, bool K1, typename C, class Ld, class St>
__device__ __forceinline__ void core_fft(const CoreDesc& d, int tpb, const SmemIO<C>& sm, const Ld& ld,
                                         const St& st) {
  const C* tw = static_cast<const C*>(d.tw);
  const StageList& sg = d.st;
  const int m = sg.n;
  if constexpr (!BLUE) {
    constexpr bool kLoad = !same_type<Ld, SmemIO<C>>::value;
    constexpr bool kStore = !same_type<St, SmemIO<C>>::value;
    if (FUSED && kLoad && kStore && sg.npass >= 2) {
      pass_any<TMINOR, K1>(sg.rf, m, 1, tpb, tw, ld, sm);
      const int Ns = smem_passes<TMINOR, K1>(sg.mid, m, sg.rf, tpb, tw, sm);
      pass_any<TMINOR, K1>(sg.rl, m, Ns, tpb, tw, sm, st);
    } else {
      if (kLoad) load_phase<TMINOR>(sm, m, tpb, ld);
      smem_passes<TMINOR, K1>(sg.all, m, 1, tpb, tw, sm);
      if (kStore) store_phase<TMINOR>(sm, m, tpb, st);
    }
  } else {
    const C* chirp = static_cast<const C*>(d.chirp);
    ChirpIn<C, Ld> l1{ld, chirp, d.n};
    ChirpOut<C, St> s2{st, chirp, d.n};
    if (FUSED && sg.npass >= 2) {
      // FFT 1: rf fused with the chirp load, then every other pass.
      int cnt[kNumRadix];
#pragma unroll
      for (int i = 0; i < kNumRadix; i++) cnt[i] = sg.mid[i] + (radix_at(i) == sg.rl ? 1 : 0);
      pass_any<TMINOR, K1>(sg.rf, m, 1, tpb, tw, l1, sm);
      smem_passes<TMINOR, K1>(cnt, m, sg.rf, tpb, tw, sm);
      spectrum_phase<TMINOR>(sm, m, tpb, static_cast<const C*>(d.bhat));
      // FFT 2: every pass but rl, then rl fused with the chirp store.
#pragma unroll
      for (int i = 0; i < kNumRadix; i++) cnt[i] = sg.mid[i] + (radix_at(i) == sg.rf ? 1 : 0);
      const int Ns = smem_passes<TMINOR, K1>(cnt, m, 1, tpb, tw, sm);
      pass_any<TMINOR, K1>(sg.rl, m, Ns, tpb, tw, sm, s2);
    } else {
      load_phase<TMINOR>(sm, m, tpb, l1);
      smem_passes<TMINOR, K1>(sg.all, m, 1, tpb, tw, sm);
      spectrum_phase<TMINOR>(sm, m, tpb, static_cast<const C*>(d.bhat));
      smem_passes<TMINOR, K1>(sg.all, m, 1, tpb, tw, sm);
      store_phase<TMINOR>(sm, d.n, tpb, s2);
    }
  }
}

// ---------------------------------------------------------------------------
// Core policies. Every transform kernel is a template over one of these:
//   DynCore  - stage list read at run time (the kernels compiled into the
//              library, one per kind / dtype / variant);
//   StatCore - stage list, lengths, sequences per CTA and tile stride fixed
//              at compile time (kernels the plan compiler emits for one plan
//              and compiles at plan time), so every index computation folds
//              to constants and each pass is straight-line code.
template <bool BLUE, bool TMINOR, bool FUSED, bool K1>
struct DynCore {
  static constexpr bool kK1 = K1;
  static constexpr bool kStatic = false;
  static constexpr int kThreads = kMaxThreads;
  static constexpr int kMinBlocks = K1 ? 2 : 1;  // launch bounds: resident CTAs per SM
  // The kernel's shared-memory tile (layout shared with the kernel's own
  // pre-/post-phases).
  template <typename C>
  __device__ __forceinline__ static SmemIO<C> tile(unsigned char* base, int ld) {
    return SmemIO<C>{reinterpret_cast<C*>(base), ld};
  }
  template <typename C, class Ld, class St>
  __device__ __forceinline__ static void run(const CoreDesc& d, int tpb, const SmemIO<C>& sm, const Ld& ld,
                                             const St& st) {
    core_fft<BLUE, TMINOR, FUSED, K1>(d, tpb, sm, ld, st);
  }
};

// Passes R, Rest... with Ns = NS at the first and this pass's stage-table
// block at stw + OFF: `ld` feeds the first pass, `st` takes the last, the
// tile carries everything in between. ROWS_FIRST maps the first pass's
// threads along each sequence (coalesced loads of contiguous rows) whatever
// TMINOR says for the others; any mapping of a pass's butterflies to threads
// computes the same transform.
// EPT > 0 (with K1 false) gives every thread EPT / R butterflies of a
// radix-R pass: EPT = the largest radix keeps every thread busy in every
// pass of a mixed-radix list.
template <int N, int TPB, int LD, int P, bool TMINOR, bool K1, int EPT, int NS, int OFF, bool ROWS_FIRST, int R,
          int... Rest, typename C, class Ld, class St>
__device__ __forceinline__ void static_passes(const C* stw, C* s, const Ld& ld, const St& st) {
  constexpr bool kMinor = TMINOR && !(ROWS_FIRST && OFF == 0);
  if constexpr (sizeof...(Rest) == 0) {
    pass_body<R, kMinor, K1, true, EPT>(N, NS, TPB, stw + OFF, ld, st);
  } else {
    const SmemIO<C, P> sm{s, LD};
    pass_body<R, kMinor, K1, true, EPT>(N, NS, TPB, stw + OFF, ld, sm);
    static_passes<N, TPB, LD, P, TMINOR, K1, EPT, NS * R, OFF + (R - 1) * NS, ROWS_FIRST, Rest...>(stw, s, sm, st);
  }
}

// Bluestein: the first FFT's last pass stores conj(Y_i * B^_i), the input of
// the inverse FFT, straight into the tile.
template <typename C, class Tile>
struct SpectrumStore {
  const Tile& sm;
  const C* bhat;
  __device__ __forceinline__ void store(int t, int i, C v) const {
    sm.store(t, i, cconj(cmul(v, __ldg(&bhat[i]))));
  }
};

// THR: the threads the kernel is launched with; MINB: the resident CTAs per
// SM its launch bounds ask for (the register budget follows from both);
// EPT: elements per thread of the several-butterflies variant (0: the
// dtype's default).
template <bool BLUE, bool TMINOR, bool K1, int M, int NU, int TPB, int LD, int P, int THR, int MINB, int EPT,
          int... Rs>
struct StatCore {
  static constexpr bool kK1 = K1;
  static constexpr bool kStatic = true;
  static constexpr int kThreads = THR;
  static constexpr int kMinBlocks = MINB;
  template <typename C>
  __device__ __forceinline__ static SmemIO<C, P> tile(unsigned char* base, int) {
    return SmemIO<C, P>{reinterpret_cast<C*>(base), LD};
  }
  // ROWS_FIRST: `ld` reads contiguous sequences, so the first pass maps
  // threads along them (the column-mapped transposing row pass).
  template <bool ROWS_FIRST = false, typename C, class Ld, class St>
  __device__ __forceinline__ static void run(const CoreDesc& d, int, const SmemIO<C, P>& sm, const Ld& ld,
                                             const St& st) {
    const C* stw = static_cast<const C*>(d.stw);
    if constexpr (!BLUE) {
      static_passes<M, TPB, LD, P, TMINOR, K1, EPT, 1, 0, ROWS_FIRST, Rs...>(stw, sm.s, ld, st);
    } else {
      const C* chirp = static_cast<const C*>(d.chirp);
      ChirpIn<C, Ld> l1{ld, chirp, NU};
      ChirpOut<C, St> s2{st, chirp, NU};
      SpectrumStore<C, SmemIO<C, P>> spec{sm, static_cast<const C*>(d.bhat)};
      static_passes<M, TPB, LD, P, TMINOR, K1, EPT, 1, 0, ROWS_FIRST, Rs...>(stw, sm.s, l1, spec);
      static_passes<M, TPB, LD, P, TMINOR, K1, EPT, 1, 0, false, Rs...>(stw, sm.s, sm, s2);
    }
  }
};

}  // namespace chfft
