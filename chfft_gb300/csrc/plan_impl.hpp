// Plan objects behind the C ABI: the five plan types of the reference,
// their tables, launch geometry and the per-method (direction, scale)
// table. Shared by the C ABI (capi.cu) and the autotuner (tune.cu).
#pragma once

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/chfft_gpu.h"
#include "cluster.hpp"
#include "jit.hpp"
#include "plan.hpp"
namespace chfft {

inline thread_local std::string tl_error;

inline int set_error(int code, const std::string& msg) {
  tl_error = msg;
  return code;
}

enum ScaleKind { S_ONE, S_UNITARY, S_N, S_DCT_U, S_DCT_N, S_MDCT_UI, S_MDCT_U };

struct MethodSpec {
  bool ok = false;
  bool back = false;
  ScaleKind scale = S_ONE;
};

// The reference's method table per type: CFft1D (src/cfft1d.rs:270-455),
// CFft2D (src/cfft2d.rs:150-321), RFft1D (src/rfft1d.rs:199-313),
// Dct1D (src/dct1d.rs:98-144), Mdct1D (src/mdct1d.rs:149-195).
inline MethodSpec method_spec(int kind, int m) {
  MethodSpec s;
  auto set = [&](bool back, ScaleKind k) {
    s.ok = true;
    s.back = back;
    s.scale = k;
  };
  switch (kind) {
    case CHFFT_KIND_CFFT1D:
    case CHFFT_KIND_CFFT2D:
    case CHFFT_KIND_CFFT3D:
    case CHFFT_KIND_RFFT1D:
      switch (m) {
        case CHFFT_FORWARD: case CHFFT_FORWARD0: set(false, S_ONE); break;
        case CHFFT_FORWARDU: set(false, S_UNITARY); break;
        case CHFFT_FORWARDN: set(false, S_N); break;
        case CHFFT_BACKWARD: set(true, S_N); break;
        case CHFFT_BACKWARD0: set(true, S_ONE); break;
        case CHFFT_BACKWARDU: set(true, S_UNITARY); break;
        case CHFFT_BACKWARDN: if (kind != CHFFT_KIND_CFFT2D && kind != CHFFT_KIND_CFFT3D) set(true, S_N); break;
        case CHFFT_FORWARD0I: if (kind == CHFFT_KIND_CFFT1D) set(false, S_ONE); break;
        case CHFFT_BACKWARD0I: if (kind == CHFFT_KIND_CFFT1D) set(true, S_ONE); break;
        case CHFFT_FORWARDUI: if (kind == CHFFT_KIND_CFFT1D) set(false, S_UNITARY); break;
        case CHFFT_BACKWARDUI: if (kind == CHFFT_KIND_CFFT1D) set(true, S_UNITARY); break;
        default: break;
      }
      break;
    case CHFFT_KIND_DCT1D:
      switch (m) {
        case CHFFT_FORWARD: case CHFFT_FORWARD0: set(false, S_ONE); break;
        case CHFFT_FORWARDU: set(false, S_DCT_U); break;
        case CHFFT_FORWARDN: set(false, S_DCT_N); break;
        default: break;
      }
      break;
    case CHFFT_KIND_MDCT1D:
      switch (m) {
        case CHFFT_FORWARD: set(false, S_MDCT_UI); break;
        case CHFFT_FORWARDU: set(false, S_ONE); break;
        case CHFFT_BACKWARD: set(true, S_MDCT_U); break;
        case CHFFT_BACKWARDU: set(true, S_ONE); break;
        default: break;
      }
      break;
    default: break;
  }
  return s;
}

struct PlanImpl {
  int kind = 0, dtype = 0;
  long long len = 0, len_m = 0, len_n = 0, len_l = 0;
  int dct_type = CHFFT_DCT_TWO;
  bool ortho = false;
  int window = CHFFT_WINDOW_SINE;
  std::vector<unsigned char> custom_window;
  Core core;   // complex core (CFft1D: N; CFft2D rows: N; RFft1D/Dct1D: N/2; Mdct1D: N/4)
  Core core2;  // CFft2D / CFft3D columns: M
  Core core3;  // CFft3D outer axis: L
  BigCore big;           // CFft1D beyond one CTA (four-step)
  bool use_big = false;
  // CFft1D of a prime length with a 7-smooth n - 1: Rader's algorithm
  // instead of Chirp-Z when CHFFT_RADER=1 (measured slower than the fused
  // Chirp-Z core on GB300: N = 1009 x 4096 66 us against 47 us; the staged
  // row doubles the shared memory per sequence). `core` still holds the
  // Chirp-Z core for the other paths.
  RaderCore rader;
  bool use_rader = false;
  // CFft1D batches of at most clus.max_batch transforms: one thread-block
  // cluster per transform (the latency form).
  ClusterCore clus;
  PlanOpts opts;         // tuning knobs (chfft_plan_set_config)
  DevBuf work;           // four-step workspace
  DevBuf aux0, aux1;
  cudaStream_t stream = nullptr;
  DevBuf stage_in, stage_out;
  // Host-memory execution pipeline: copy-in and copy-out streams and one
  // event pair per chunk.
  static constexpr int kMaxChunks = 8;
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  cudaEvent_t ev_in[kMaxChunks] = {}, ev_done[kMaxChunks] = {};

  ~PlanImpl() {
    for (int k = 0; k < kMaxChunks; k++) {
      if (ev_in[k]) cudaEventDestroy(ev_in[k]);
      if (ev_done[k]) cudaEventDestroy(ev_done[k]);
    }
    if (copy_in) cudaStreamDestroy(copy_in);
    if (copy_out) cudaStreamDestroy(copy_out);
    if (stream) cudaStreamDestroy(stream);
  }

  cudaStream_t host_stream() {
    if (!stream) CHFFT_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    return stream;
  }

  // (Re)build every table for the current lengths. Returns a status.
  int build() {
    cudaStream_t s = host_stream();
    aux0.release();
    aux1.release();
    const size_t cb = cplx_bytes(dtype), rb = real_bytes(dtype);
    auto gen = [&](Table t, long long n, long long count, void* out) {
      CHFFT_CUDA(dtype == 0 ? gen_table<float>(t, n, count, 0, out, s) : gen_table<double>(t, n, count, 0, out, s));
    };
    auto need = [&](Core& c, long long n) {
      if (!c.build(n, dtype, s, opts.blue_m)) throw Fail{CHFFT_EUNSUPPORTED, "transform length " + std::to_string(n) + " exceeds the shared-memory engine"};
    };
    use_big = false;
    switch (kind) {
      case CHFFT_KIND_CFFT1D: {
        use_rader = false;
        rader.release();
        const bool one_cta = len < 2 || core.build(len, dtype, s, opts.blue_m);
        if (len >= 2 && (!one_cta || core.blue)) {
          // A prime length: Rader when its n - 1 core fits one CTA.
          const char* e = std::getenv("CHFFT_RADER");
          if (e && e[0] == '1' && opts.blue_m == 0) use_rader = rader.build(len, dtype, s);
        }
        if (!one_cta && !use_rader) {
          if (!big.build(len, dtype, s, opts))
            throw Fail{CHFFT_EUNSUPPORTED, "transform length " + std::to_string(len) + " is not supported"};
          use_big = true;
        }
        clus.release();
        if (!use_rader && !(one_cta && core.blue) && !(use_big && big.blue)) clus.build(len, dtype, s, use_big);
        break;
      }
      case CHFFT_KIND_CFFT2D:
        if (len_m > 0 && len_n > 0) {
          need(core, len_n);
          need(core2, len_m);
        }
        break;
      case CHFFT_KIND_CFFT3D:
        if (len_l > 0 && len_m > 0 && len_n > 0) {
          need(core, len_n);
          need(core2, len_m);
          need(core3, len_l);
        }
        break;
      case CHFFT_KIND_RFFT1D: {
        long long h = len / 2;
        need(core, h);
        aux0.ensure(h * cb);
        aux1.ensure(h * cb);
        gen(Table::RCOEF, len, h, aux0.p);
        gen(Table::RBCOEF, len, h, aux1.p);
        // small batches: the half-length FFT on a cluster, split / merge apart
        clus.release();
        if (!core.blue) clus.build(h, dtype, s);
        break;
      }
      case CHFFT_KIND_DCT1D: {
        long long h = len / 2;
        need(core, h);
        aux0.ensure(h * cb);
        aux1.ensure((h + 1) * cb);
        gen(dct_type == CHFFT_DCT_TWO ? Table::RCOEF : Table::RBCOEF, len, h, aux0.p);
        gen(dct_type == CHFFT_DCT_TWO ? Table::OMEGA4N_POS : Table::OMEGA4N_NEG, len, h + 1, aux1.p);
        clus.release();
        if (!core.blue) clus.build(h, dtype, s);
        break;
      }
      case CHFFT_KIND_MDCT1D: {
        long long q = len / 4;
        need(core, q);
        aux0.ensure(q * cb);
        aux1.ensure(len * rb);
        gen(Table::MDCT_TW, len, q, aux0.p);
        if (window == CHFFT_WINDOW_CUSTOM)
          CHFFT_CUDA(cudaMemcpyAsync(aux1.p, custom_window.data(), len * rb, cudaMemcpyHostToDevice, s));
        else
          gen(window == CHFFT_WINDOW_VORBIS ? Table::VORBIS_WIN : Table::SINE_WIN, len, len, aux1.p);
        clus.release();
        if (!core.blue) clus.build(q, dtype, s);
        break;
      }
    }
    CHFFT_CUDA(cudaStreamSynchronize(s));
    return CHFFT_OK;
  }

  // Applies tuning knobs; the tables are rebuilt when the Bluestein length
  // or the four-step split changes.
  void apply(const PlanOpts& o) {
    const bool rebuild = o.blue_m != opts.blue_m || o.fs_n1 != opts.fs_n1;  // (also decides Rader vs Chirp-Z)
    opts = o;
    big.opts = o;
    if (rebuild) build();
  }

  // Elements (of the side's own type) per transform for a method direction.
  size_t in_elems(bool back) const {
    switch (kind) {
      case CHFFT_KIND_CFFT1D: return (size_t)len;
      case CHFFT_KIND_CFFT2D: return (size_t)(len_m * len_n);
      case CHFFT_KIND_CFFT3D: return (size_t)(len_l * len_m * len_n);
      case CHFFT_KIND_RFFT1D: return back ? (size_t)(len / 2 + 1) : (size_t)len;
      case CHFFT_KIND_DCT1D: return (size_t)len;
      default: return back ? (size_t)(len / 2) : (size_t)len;
    }
  }
  size_t out_elems(bool back) const {
    switch (kind) {
      case CHFFT_KIND_RFFT1D: return back ? (size_t)len : (size_t)(len / 2 + 1);
      case CHFFT_KIND_MDCT1D: return back ? (size_t)len : (size_t)(len / 2);
      default: return in_elems(back);
    }
  }
  // Bytes per element of the input / output side.
  size_t in_esize(bool back) const {
    switch (kind) {
      case CHFFT_KIND_CFFT1D: case CHFFT_KIND_CFFT2D: case CHFFT_KIND_CFFT3D: return cplx_bytes(dtype);
      case CHFFT_KIND_RFFT1D: return back ? cplx_bytes(dtype) : real_bytes(dtype);
      default: return real_bytes(dtype);
    }
  }
  size_t out_esize(bool back) const {
    if (kind == CHFFT_KIND_RFFT1D) return back ? real_bytes(dtype) : cplx_bytes(dtype);
    return in_esize(back);
  }

  double scale_value(ScaleKind k) const {
    double n = kind == CHFFT_KIND_CFFT2D   ? (double)len_m * (double)len_n
               : kind == CHFFT_KIND_CFFT3D ? (double)len_l * (double)len_m * (double)len_n
                                           : (double)len;
    switch (k) {
      case S_ONE: return 1.0;
      case S_UNITARY: return 1.0 / std::sqrt(n);
      case S_N: return 1.0 / n;
      case S_DCT_U: return std::sqrt(2.0 / n);
      case S_DCT_N: return 2.0 / n;
      case S_MDCT_UI: return std::sqrt(n / 2.0);
      case S_MDCT_U: return 1.0 / std::sqrt(n / 2.0);
    }
    return 1.0;
  }

  // Plan-time specialised kernel when the plan compiler is on for this batch
  // size (CHFFT_JIT: auto = batches of >= 2^18 elements), else the library
  // kernel with run-time stages.
  template <typename T>
  void dispatch(Kernel k, const Core& c, const Geo& g, const KArgs& a, unsigned blocks, long long elems,
                cudaStream_t s) {
    const bool want = c.st.n > 1 && want_specialised(elems, opts.jit);
    if (want) {
      int r = jit_launch(k, dtype, c, g, a, blocks, s);
      if (r == 0) return;
      if (r == 2) throw Fail{CHFFT_ECUDA, "launch of a plan-time specialised kernel failed"};
    }
    CHFFT_CUDA(launch_kernel<T>(k, c.blue, g.k1, a, blocks, g.threads, g.smem, s));
  }

  template <typename T>
  void launch(Kernel k, const Core& c, KArgs& a, long long count, cudaStream_t s) {
    if (opts.tc > 0) {
      // Radix-16 passes on the tensor cores: plain f32 C2C rows only.
      if (k != Kernel::C2C || dtype != CHFFT_F32 || c.blue || c.tc_s16 < 1)
        throw Fail{CHFFT_EUNSUPPORTED, "tensor-core passes need an f32 CFft1D plan of power-of-two length >= 16"};
      int tpb = (int)std::max<long long>(1, 4096 / c.st.n);
      a.core = c.desc();
      a.count = count;
      const unsigned blocks = (unsigned)((count + tpb - 1) / tpb);
      const int r = jit_launch_tc(k, c, opts.tc, tpb, a, blocks, s);
      if (r == 2) throw Fail{CHFFT_ECUDA, "launch of a tensor-core kernel failed"};
      if (r == 1) throw Fail{CHFFT_EUNSUPPORTED, "tensor-core kernel unavailable (plan compiler or geometry)"};
      return;
    }
    Geo g = row_geo(c, count, opts);
    a.core = c.desc();
    a.tpb = g.tpb;
    a.ld = g.ld;
    a.count = count;
    unsigned blocks = (unsigned)((count + g.tpb - 1) / g.tpb);
    dispatch<T>(k, c, g, a, blocks, count * c.n, s);
  }

  template <typename T>
  void launch_rader(KArgs& a, long long count, cudaStream_t s) {
    int ldr = 0;
    Geo g = rader_geo(rader, count, opts, &ldr);
    a.core = rader.lc.desc();
    a.tpb = g.tpb;
    a.ld = g.ld;
    a.count = count;
    a.aux0 = rader.perm.p;
    a.aux1 = rader.bhat.p;
    a.n_user = (int)rader.n;
    a.ncols = ldr;
    const unsigned blocks = (unsigned)((count + g.tpb - 1) / g.tpb);
    dispatch<T>(Kernel::C2C_RADER, rader.lc, g, a, blocks, count * rader.n, s);
  }

  template <typename T>
  void exec_t(const MethodSpec& ms, const void* d_in, void* d_out, long long batch, cudaStream_t s) {
    const double sc = scale_value(ms.scale);
    KArgs a{};
    a.in = d_in;
    a.out = d_out;
    a.scale = sc;
    a.back = ms.back ? 1 : 0;
    switch (kind) {
      case CHFFT_KIND_CFFT1D:
        if (len <= 1) {  // chfft returns a copy for len <= 1 (src/cfft1d.rs:212-214)
          if (d_in != d_out && len == 1)
            CHFFT_CUDA(cudaMemcpyAsync(d_out, d_in, batch * cplx_bytes(dtype), cudaMemcpyDeviceToDevice, s));
          return;
        }
        if (clus.n && batch <= clus.max_batch && opts.tc <= 0 && clus.exec(d_in, d_out, batch, ms.back, sc, s))
          return;
        if (use_big) {
          work.ensure((size_t)big.work_elems(batch) * cplx_bytes(dtype));
          big.exec(d_in, d_out, work.p, batch, ms.back, sc, s);
          return;
        }
        a.in_dist = a.out_dist = len;
        if (use_rader && opts.tc <= 0) {
          launch_rader<T>(a, batch, s);
          return;
        }
        launch<T>(Kernel::C2C, core, a, batch, s);
        return;
      case CHFFT_KIND_CFFT2D: {
        if (len_m == 0 || len_n == 0) return;
        // Row FFTs of length N into d_out, then column FFTs of length M in
        // place with the scale (src/cfft2d.rs:340-361).
        a.in_dist = a.out_dist = len_n;
        a.scale = 1.0;
        launch<T>(Kernel::C2C, core, a, batch * len_m, s);
        KArgs b{};
        b.core = core2.desc();
        Geo g = col_geo(core2, (int)len_n, opts.fs_tpb, opts);
        b.tpb = g.tpb;
        b.ld = g.ld;
        b.back = a.back;
        b.count = batch;
        b.tiles_per_tr = (len_n + g.tpb - 1) / g.tpb;
        b.in = d_out;
        b.out = d_out;
        b.scale = sc;
        b.in_dist = b.out_dist = len_m * len_n;
        b.ncols = (int)len_n;
        dispatch<T>(Kernel::COLS, core2, g, b, (unsigned)(batch * b.tiles_per_tr), batch * len_m * len_n, s);
        return;
      }
      case CHFFT_KIND_CFFT3D: {
        if (len_l == 0 || len_m == 0 || len_n == 0) return;
        // Rows of N into d_out, then the M axis (column tiles of each of the
        // batch x L planes, in place), then the L axis (column tiles over
        // the M x N columns of each volume, in place, with the scale).
        a.in_dist = a.out_dist = len_n;
        a.scale = 1.0;
        launch<T>(Kernel::C2C, core, a, batch * len_l * len_m, s);
        auto columns = [&](const Core& c, long long count, long long ncols, long long rows, double scale) {
          KArgs b{};
          b.core = c.desc();
          Geo g = col_geo(c, (int)ncols, opts.fs_tpb, opts);
          b.tpb = g.tpb;
          b.ld = g.ld;
          b.back = a.back;
          b.count = count;
          b.tiles_per_tr = (ncols + g.tpb - 1) / g.tpb;
          b.in = d_out;
          b.out = d_out;
          b.scale = scale;
          b.in_dist = b.out_dist = rows * ncols;
          b.ncols = (int)ncols;
          dispatch<T>(Kernel::COLS, c, g, b, (unsigned)(count * b.tiles_per_tr), count * rows * ncols, s);
        };
        columns(core2, batch * len_l, len_n, len_m, 1.0);
        columns(core3, batch, len_m * len_n, len_l, sc);
        return;
      }
      case CHFFT_KIND_RFFT1D:
        if (clus.n && batch <= clus.max_batch && opts.tc <= 0) {
          // The half-length FFT on a cluster with scale 1, the split (forward)
          // or the merge (backward, times 2 scale) in its own launch.
          const int h = (int)(len / 2);
          work.ensure((size_t)batch * h * cplx_bytes(dtype));
          if (!ms.back) {
            if (clus.exec(d_in, work.p, batch, false, 1.0, s)) {
              CHFFT_CUDA(rfft_split(dtype, work.p, d_out, aux0.p, h, batch, sc, s));
              return;
            }
          } else {
            CHFFT_CUDA(rfft_merge(dtype, d_in, work.p, aux1.p, h, batch, 2.0 * sc, s));
            if (clus.exec(work.p, d_out, batch, true, 1.0, s)) return;
          }
        }
        a.aux0 = ms.back ? aux1.p : aux0.p;
        a.in_dist = ms.back ? len / 2 + 1 : len;
        a.out_dist = ms.back ? len : len / 2 + 1;
        launch<T>(ms.back ? Kernel::C2R : Kernel::R2C, core, a, batch, s);
        return;
      case CHFFT_KIND_DCT1D:
        a.aux0 = aux0.p;
        a.aux1 = aux1.p;
        a.in_dist = a.out_dist = len;
        // ortho: x0 * sqrt(1/2) (DCT-II) or 1/2 -> sqrt(1/2) (DCT-III) (src/dct1d.rs:220-224, :343-347)
        a.aux_scalar = ortho ? std::sqrt(0.5) : (dct_type == CHFFT_DCT_TWO ? 1.0 : 0.5);
        if (clus.n && batch <= clus.max_batch && opts.tc <= 0) {
          // The half-length FFT on a cluster (scale 1, in place on the
          // workspace) between the pre-twiddle / packing and the post launch;
          // DCT-III's core runs backward on the unconjugated merge.
          const int op = dct_type == CHFFT_DCT_TWO ? kDct2 : kDct3;
          work.ensure((size_t)batch * (len / 2) * cplx_bytes(dtype));
          CHFFT_CUDA(real_pre(dtype, op, d_in, work.p, aux0.p, aux1.p, (int)len, batch, sc, a.aux_scalar, s));
          if (clus.exec(work.p, work.p, batch, op == kDct3, 1.0, s)) {
            CHFFT_CUDA(real_post(dtype, op, work.p, d_out, aux0.p, aux1.p, (int)len, batch, sc, s));
            return;
          }
        }
        launch<T>(dct_type == CHFFT_DCT_TWO ? Kernel::DCT2 : Kernel::DCT3, core, a, batch, s);
        return;
      case CHFFT_KIND_MDCT1D:
        a.aux0 = aux0.p;
        a.aux1 = aux1.p;
        a.n_user = (int)len;
        a.in_dist = ms.back ? len / 2 : len;
        a.out_dist = ms.back ? len : len / 2;
        if (clus.n && batch <= clus.max_batch && opts.tc <= 0) {
          // The quarter-length forward FFT on a cluster (in place on the
          // workspace) between the fold / pre-twiddle and the post launch.
          const int op = ms.back ? kImdct : kMdct;
          work.ensure((size_t)batch * (len / 4) * cplx_bytes(dtype));
          CHFFT_CUDA(real_pre(dtype, op, d_in, work.p, aux0.p, aux1.p, (int)len, batch, sc, 1.0, s));
          if (clus.exec(work.p, work.p, batch, false, 1.0, s)) {
            CHFFT_CUDA(real_post(dtype, op, work.p, d_out, aux0.p, aux1.p, (int)len, batch, sc, s));
            return;
          }
        }
        launch<T>(ms.back ? Kernel::IMDCT : Kernel::MDCT, core, a, batch, s);
        return;
    }
  }

  // CFft1D on split-complex device arrays (re / im separate): the one-CTA
  // row kernels (library form). Plans beyond one CTA or on Rader's path
  // are refused.
  void exec_split(const MethodSpec& ms, const void* in_re, const void* in_im, void* out_re, void* out_im,
                  long long batch, cudaStream_t s) {
    if (kind != CHFFT_KIND_CFFT1D || use_big || use_rader || len < 2)
      throw Fail{CHFFT_EUNSUPPORTED, "split-complex execution needs a CFft1D plan of 2 or more points within one CTA"};
    if (batch <= 0) return;
    KArgs a{};
    a.in = in_re;
    a.aux0 = in_im;
    a.out = out_re;
    a.aux1 = out_im;
    a.scale = scale_value(ms.scale);
    a.back = ms.back ? 1 : 0;
    a.in_dist = a.out_dist = len;
    Geo g = row_geo(core, batch, opts);
    a.core = core.desc();
    a.tpb = g.tpb;
    a.ld = g.ld;
    a.count = batch;
    const unsigned blocks = (unsigned)((batch + g.tpb - 1) / g.tpb);
    if (dtype == CHFFT_F32)
      CHFFT_CUDA(launch_kernel<float>(Kernel::C2C_SPLIT, core.blue, g.k1, a, blocks, g.threads, g.smem, s));
    else
      CHFFT_CUDA(launch_kernel<double>(Kernel::C2C_SPLIT, core.blue, g.k1, a, blocks, g.threads, g.smem, s));
  }

  // CFft1D on strided device layouts: element i of transform t at
  // t * dist + i * stride (complex elements, input and output apart), the
  // one-CTA row kernels (library form).
  void exec_strided(const MethodSpec& ms, const void* in, long long istride, long long idist, void* out,
                    long long ostride, long long odist, long long batch, cudaStream_t s) {
    if (kind != CHFFT_KIND_CFFT1D || use_big || use_rader || len < 2)
      throw Fail{CHFFT_EUNSUPPORTED, "strided execution needs a CFft1D plan of 2 or more points within one CTA"};
    if (istride < 1 || ostride < 1 || istride > INT_MAX || ostride > INT_MAX || idist < 0 || odist < 0)
      throw Fail{CHFFT_EINVAL, "strides must be in [1, 2^31) and distances non-negative"};
    if (batch <= 0) return;
    KArgs a{};
    a.in = in;
    a.out = out;
    a.ncols = (int)istride;
    a.n_user = (int)ostride;
    a.in_dist = idist;
    a.out_dist = odist;
    a.scale = scale_value(ms.scale);
    a.back = ms.back ? 1 : 0;
    Geo g = row_geo(core, batch, opts);
    a.core = core.desc();
    a.tpb = g.tpb;
    a.ld = g.ld;
    a.count = batch;
    const unsigned blocks = (unsigned)((batch + g.tpb - 1) / g.tpb);
    if (dtype == CHFFT_F32)
      CHFFT_CUDA(launch_kernel<float>(Kernel::C2C_STRIDED, core.blue, g.k1, a, blocks, g.threads, g.smem, s));
    else
      CHFFT_CUDA(launch_kernel<double>(Kernel::C2C_STRIDED, core.blue, g.k1, a, blocks, g.threads, g.smem, s));
  }

  // Throws CHFFT_ETIMEOUT when a bounded device-side wait of this plan's
  // kernels gave up since the last check (the host-mapped word the
  // pipelined four-step launch sets). Call after a synchronisation.
  void check_waits() {
    if (int code = big.err.take())
      throw Fail{CHFFT_ETIMEOUT, "a device-side wait of the pipelined four-step launch gave up (code " +
                                     std::to_string(code) + "); that launch's output is incomplete"};
    if (int code = clus.err.take())
      throw Fail{CHFFT_ETIMEOUT, "a CTA of the cluster launch gave up waiting for its rows (code " +
                                     std::to_string(code) + "); that launch's output is incomplete"};
  }

  void exec(const MethodSpec& ms, const void* d_in, void* d_out, long long batch, cudaStream_t s) {
    if (batch <= 0) return;
    if (dtype == CHFFT_F32)
      exec_t<float>(ms, d_in, d_out, batch, s);
    else
      exec_t<double>(ms, d_in, d_out, batch, s);
  }

  // Host memory: stage in, run, stage out, synchronise. Batches of more
  // than 8 MiB run as a pipeline of up to kMaxChunks chunks: the copy-in of
  // chunk k+1, the transforms of chunk k and the copy-out of chunk k-1
  // overlap (copy engines of both directions and the SMs); with pinned host
  // memory the end-to-end time approaches the larger of the two copies.
  void exec_host(const MethodSpec& ms, const void* src, void* dst, long long batch) {
    cudaStream_t s = host_stream();
    const size_t ib1 = in_elems(ms.back) * in_esize(ms.back), ob1 = out_elems(ms.back) * out_esize(ms.back);
    const size_t ib = ib1 * batch, ob = ob1 * batch;
    if (ib == 0 && ob == 0) return;
    stage_in.ensure(ib);
    stage_out.ensure(ob);
    const long long chunks =
        std::max(1LL, std::min<long long>({batch, (long long)kMaxChunks, (long long)((ib + ob) >> 23)}));
    if (chunks == 1 || ib1 == 0 || ob1 == 0) {
      if (ib) CHFFT_CUDA(cudaMemcpyAsync(stage_in.p, src, ib, cudaMemcpyHostToDevice, s));
      exec(ms, stage_in.p, stage_out.p, batch, s);
      if (ob) CHFFT_CUDA(cudaMemcpyAsync(dst, stage_out.p, ob, cudaMemcpyDeviceToHost, s));
      CHFFT_CUDA(cudaStreamSynchronize(s));
      check_waits();
      return;
    }
    if (!copy_in) CHFFT_CUDA(cudaStreamCreateWithFlags(&copy_in, cudaStreamNonBlocking));
    if (!copy_out) CHFFT_CUDA(cudaStreamCreateWithFlags(&copy_out, cudaStreamNonBlocking));
    for (int k = 0; k < kMaxChunks; k++) {
      if (!ev_in[k]) CHFFT_CUDA(cudaEventCreateWithFlags(&ev_in[k], cudaEventDisableTiming));
      if (!ev_done[k]) CHFFT_CUDA(cudaEventCreateWithFlags(&ev_done[k], cudaEventDisableTiming));
    }
    const long long per = (batch + chunks - 1) / chunks;
    const char* hs = static_cast<const char*>(src);
    char* hd = static_cast<char*>(dst);
    char* di = static_cast<char*>(stage_in.p);
    char* dout = static_cast<char*>(stage_out.p);
    int k = 0;
    for (long long c0 = 0; c0 < batch; c0 += per, k++) {
      const long long cnt = std::min(per, batch - c0);
      CHFFT_CUDA(cudaMemcpyAsync(di + c0 * ib1, hs + c0 * ib1, cnt * ib1, cudaMemcpyHostToDevice, copy_in));
      CHFFT_CUDA(cudaEventRecord(ev_in[k], copy_in));
      CHFFT_CUDA(cudaStreamWaitEvent(s, ev_in[k], 0));
      exec(ms, di + c0 * ib1, dout + c0 * ob1, cnt, s);
      CHFFT_CUDA(cudaEventRecord(ev_done[k], s));
      CHFFT_CUDA(cudaStreamWaitEvent(copy_out, ev_done[k], 0));
      CHFFT_CUDA(cudaMemcpyAsync(hd + c0 * ob1, dout + c0 * ob1, cnt * ob1, cudaMemcpyDeviceToHost, copy_out));
    }
    CHFFT_CUDA(cudaStreamSynchronize(copy_out));
    CHFFT_CUDA(cudaStreamSynchronize(s));
    check_waits();
  }
};

}  // namespace chfft

struct chfft_plan_s {
  chfft::PlanImpl impl;
};
