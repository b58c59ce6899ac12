// The C ABI (include/chfft_gpu.h): plan objects mirroring chfft's five plan
// types, their setup methods and the per-method (direction, scale) table.
#include <cmath>
#include <cstring>
#include <functional>
#include <new>
#include <string>
#include <vector>

#include "../../include/chfft_gpu.h"
#include "jit.hpp"
#include "plan.hpp"

namespace chfft {
namespace {

thread_local std::string tl_error;

int set_error(int code, const std::string& msg) {
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
MethodSpec method_spec(int kind, int m) {
  MethodSpec s;
  auto set = [&](bool back, ScaleKind k) {
    s.ok = true;
    s.back = back;
    s.scale = k;
  };
  switch (kind) {
    case CHFFT_KIND_CFFT1D:
    case CHFFT_KIND_CFFT2D:
    case CHFFT_KIND_RFFT1D:
      switch (m) {
        case CHFFT_FORWARD: case CHFFT_FORWARD0: set(false, S_ONE); break;
        case CHFFT_FORWARDU: set(false, S_UNITARY); break;
        case CHFFT_FORWARDN: set(false, S_N); break;
        case CHFFT_BACKWARD: set(true, S_N); break;
        case CHFFT_BACKWARD0: set(true, S_ONE); break;
        case CHFFT_BACKWARDU: set(true, S_UNITARY); break;
        case CHFFT_BACKWARDN: if (kind != CHFFT_KIND_CFFT2D) set(true, S_N); break;
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

}  // namespace

struct PlanImpl {
  int kind = 0, dtype = 0;
  long long len = 0, len_m = 0, len_n = 0;
  int dct_type = CHFFT_DCT_TWO;
  bool ortho = false;
  int window = CHFFT_WINDOW_SINE;
  std::vector<unsigned char> custom_window;
  Core core;   // complex core (CFft1D: N; CFft2D rows: N; RFft1D/Dct1D: N/2; Mdct1D: N/4)
  Core core2;  // CFft2D columns: M
  BigCore big;           // CFft1D beyond one CTA (four-step)
  bool use_big = false;
  DevBuf work;           // four-step workspace
  DevBuf aux0, aux1;
  cudaStream_t stream = nullptr;
  DevBuf stage_in, stage_out;

  ~PlanImpl() {
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
      if (!c.build(n, dtype, s)) throw Fail{CHFFT_EUNSUPPORTED, "transform length " + std::to_string(n) + " exceeds the shared-memory engine"};
    };
    use_big = false;
    switch (kind) {
      case CHFFT_KIND_CFFT1D:
        if (len >= 2 && !core.build(len, dtype, s)) {
          if (!big.build(len, dtype, s))
            throw Fail{CHFFT_EUNSUPPORTED, "transform length " + std::to_string(len) + " is not supported"};
          use_big = true;
        }
        break;
      case CHFFT_KIND_CFFT2D:
        if (len_m > 0 && len_n > 0) {
          need(core, len_n);
          need(core2, len_m);
        }
        break;
      case CHFFT_KIND_RFFT1D: {
        long long h = len / 2;
        need(core, h);
        aux0.ensure(h * cb);
        aux1.ensure(h * cb);
        gen(Table::RCOEF, len, h, aux0.p);
        gen(Table::RBCOEF, len, h, aux1.p);
        break;
      }
      case CHFFT_KIND_DCT1D: {
        long long h = len / 2;
        need(core, h);
        aux0.ensure(h * cb);
        aux1.ensure((h + 1) * cb);
        gen(dct_type == CHFFT_DCT_TWO ? Table::RCOEF : Table::RBCOEF, len, h, aux0.p);
        gen(dct_type == CHFFT_DCT_TWO ? Table::OMEGA4N_POS : Table::OMEGA4N_NEG, len, h + 1, aux1.p);
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
        break;
      }
    }
    CHFFT_CUDA(cudaStreamSynchronize(s));
    return CHFFT_OK;
  }

  // Elements (of the side's own type) per transform for a method direction.
  size_t in_elems(bool back) const {
    switch (kind) {
      case CHFFT_KIND_CFFT1D: return (size_t)len;
      case CHFFT_KIND_CFFT2D: return (size_t)(len_m * len_n);
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
      case CHFFT_KIND_CFFT1D: case CHFFT_KIND_CFFT2D: return cplx_bytes(dtype);
      case CHFFT_KIND_RFFT1D: return back ? cplx_bytes(dtype) : real_bytes(dtype);
      default: return real_bytes(dtype);
    }
  }
  size_t out_esize(bool back) const {
    if (kind == CHFFT_KIND_RFFT1D) return back ? real_bytes(dtype) : cplx_bytes(dtype);
    return in_esize(back);
  }

  double scale_value(ScaleKind k) const {
    double n = kind == CHFFT_KIND_CFFT2D ? (double)len_m * (double)len_n : (double)len;
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
    const JitMode mode = jit_mode();
    const bool want = c.st.n > 1 && (mode == JitMode::ALWAYS || (mode == JitMode::AUTO && elems >= (1LL << 18)));
    if (want) {
      int r = jit_launch(k, dtype, c, g, a, blocks, s);
      if (r == 0) return;
      if (r == 2) throw Fail{CHFFT_ECUDA, "launch of a plan-time specialised kernel failed"};
    }
    CHFFT_CUDA(launch_kernel<T>(k, c.blue, g.k1, a, blocks, g.threads, g.smem, s));
  }

  template <typename T>
  void launch(Kernel k, const Core& c, KArgs& a, long long count, cudaStream_t s) {
    Geo g = row_geo(c, count);
    a.core = c.desc();
    a.tpb = g.tpb;
    a.ld = g.ld;
    a.count = count;
    unsigned blocks = (unsigned)((count + g.tpb - 1) / g.tpb);
    dispatch<T>(k, c, g, a, blocks, count * c.n, s);
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
        if (use_big) {
          work.ensure((size_t)big.work_elems(batch) * cplx_bytes(dtype));
          big.exec(d_in, d_out, work.p, batch, ms.back, sc, s);
          return;
        }
        a.in_dist = a.out_dist = len;
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
        Geo g = col_geo(core2, (int)len_n);
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
      case CHFFT_KIND_RFFT1D:
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
        launch<T>(dct_type == CHFFT_DCT_TWO ? Kernel::DCT2 : Kernel::DCT3, core, a, batch, s);
        return;
      case CHFFT_KIND_MDCT1D:
        a.aux0 = aux0.p;
        a.aux1 = aux1.p;
        a.n_user = (int)len;
        a.in_dist = ms.back ? len / 2 : len;
        a.out_dist = ms.back ? len : len / 2;
        launch<T>(ms.back ? Kernel::IMDCT : Kernel::MDCT, core, a, batch, s);
        return;
    }
  }

  void exec(const MethodSpec& ms, const void* d_in, void* d_out, long long batch, cudaStream_t s) {
    if (batch <= 0) return;
    if (dtype == CHFFT_F32)
      exec_t<float>(ms, d_in, d_out, batch, s);
    else
      exec_t<double>(ms, d_in, d_out, batch, s);
  }

  // Host memory: stage in, run, stage out, synchronise.
  void exec_host(const MethodSpec& ms, const void* src, void* dst, long long batch) {
    cudaStream_t s = host_stream();
    const size_t ib = in_elems(ms.back) * in_esize(ms.back) * batch;
    const size_t ob = out_elems(ms.back) * out_esize(ms.back) * batch;
    if (ib == 0 && ob == 0) return;
    stage_in.ensure(ib);
    stage_out.ensure(ob);
    if (ib) CHFFT_CUDA(cudaMemcpyAsync(stage_in.p, src, ib, cudaMemcpyHostToDevice, s));
    exec(ms, stage_in.p, stage_out.p, batch, s);
    if (ob) CHFFT_CUDA(cudaMemcpyAsync(dst, stage_out.p, ob, cudaMemcpyDeviceToHost, s));
    CHFFT_CUDA(cudaStreamSynchronize(s));
  }
};

}  // namespace chfft

using chfft::Fail;
using chfft::PlanImpl;

struct chfft_plan_s {
  PlanImpl impl;
};

namespace {

template <class F>
int guarded(F&& f) {
  try {
    chfft::tl_error.clear();
    return f();
  } catch (const Fail& e) {
    return chfft::set_error(e.code, e.msg);
  } catch (const std::bad_alloc&) {
    return chfft::set_error(CHFFT_ENOMEM, "host allocation failed");
  } catch (const std::exception& e) {
    return chfft::set_error(CHFFT_EINVAL, e.what());
  }
}

bool valid_dtype(int d) { return d == CHFFT_F32 || d == CHFFT_F64; }

int create(chfft_plan* out, const std::function<int(PlanImpl&)>& init) {
  if (!out) return chfft::set_error(CHFFT_EINVAL, "null plan pointer");
  *out = nullptr;
  return guarded([&]() -> int {
    auto* p = new chfft_plan_s();
    int rc = CHFFT_OK;
    try {
      rc = init(p->impl);
      if (rc == CHFFT_OK) rc = p->impl.build();
    } catch (...) {
      delete p;
      throw;
    }
    if (rc != CHFFT_OK) {
      delete p;
      return rc;
    }
    *out = p;
    return CHFFT_OK;
  });
}

}  // namespace

extern "C" {

int chfft_cfft1d_create(int dtype, size_t len, chfft_plan* out) {
  if (!valid_dtype(dtype)) return chfft::set_error(CHFFT_EINVAL, "unknown dtype");
  return create(out, [&](PlanImpl& p) -> int {
    p.kind = CHFFT_KIND_CFFT1D;
    p.dtype = dtype;
    p.len = (long long)len;
    return CHFFT_OK;
  });
}

int chfft_cfft2d_create(int dtype, size_t len_m, size_t len_n, chfft_plan* out) {
  if (!valid_dtype(dtype)) return chfft::set_error(CHFFT_EINVAL, "unknown dtype");
  return create(out, [&](PlanImpl& p) -> int {
    p.kind = CHFFT_KIND_CFFT2D;
    p.dtype = dtype;
    p.len_m = (long long)len_m;
    p.len_n = (long long)len_n;
    p.len = p.len_m * p.len_n;
    return CHFFT_OK;
  });
}

int chfft_rfft1d_create(int dtype, size_t len, chfft_plan* out) {
  if (!valid_dtype(dtype)) return chfft::set_error(CHFFT_EINVAL, "unknown dtype");
  if ((len & 1) || len == 0) return chfft::set_error(CHFFT_EINVAL_LEN, "invalid length");
  return create(out, [&](PlanImpl& p) -> int {
    p.kind = CHFFT_KIND_RFFT1D;
    p.dtype = dtype;
    p.len = (long long)len;
    return CHFFT_OK;
  });
}

int chfft_dct1d_create(int dtype, int dct_type, size_t len, int is_ortho, chfft_plan* out) {
  if (!valid_dtype(dtype)) return chfft::set_error(CHFFT_EINVAL, "unknown dtype");
  if (dct_type != CHFFT_DCT_TWO && dct_type != CHFFT_DCT_THREE) return chfft::set_error(CHFFT_EINVAL, "unknown DCT type");
  if ((len & 1) || len == 0) return chfft::set_error(CHFFT_EINVAL_LEN, "invalid length");
  return create(out, [&](PlanImpl& p) -> int {
    p.kind = CHFFT_KIND_DCT1D;
    p.dtype = dtype;
    p.dct_type = dct_type;
    p.ortho = is_ortho != 0;
    p.len = (long long)len;
    return CHFFT_OK;
  });
}

int chfft_mdct1d_create(int dtype, size_t len, int window, const void* window_table, chfft_plan* out) {
  if (!valid_dtype(dtype)) return chfft::set_error(CHFFT_EINVAL, "unknown dtype");
  if (window < CHFFT_WINDOW_SINE || window > CHFFT_WINDOW_CUSTOM) return chfft::set_error(CHFFT_EINVAL, "unknown window");
  if (window == CHFFT_WINDOW_CUSTOM && !window_table) return chfft::set_error(CHFFT_EINVAL, "custom window needs a table");
  if ((len & 3) || len == 0) return chfft::set_error(CHFFT_EINVAL_LEN, "invalid length");
  return create(out, [&](PlanImpl& p) -> int {
    p.kind = CHFFT_KIND_MDCT1D;
    p.dtype = dtype;
    p.window = window;
    p.len = (long long)len;
    if (window == CHFFT_WINDOW_CUSTOM) {
      const auto* w = static_cast<const unsigned char*>(window_table);
      p.custom_window.assign(w, w + len * chfft::real_bytes(dtype));
    }
    return CHFFT_OK;
  });
}

int chfft_plan_destroy(chfft_plan plan) {
  delete plan;
  return CHFFT_OK;
}

int chfft_plan_setup(chfft_plan plan, size_t len, const void* window_table) {
  if (!plan) return chfft::set_error(CHFFT_EINVAL, "null plan");
  PlanImpl& p = plan->impl;
  return guarded([&]() -> int {
    switch (p.kind) {
      case CHFFT_KIND_CFFT1D: break;
      case CHFFT_KIND_RFFT1D:
        if ((len & 1) || len == 0) return chfft::set_error(CHFFT_EINVAL_LEN, "invalid length");
        break;
      case CHFFT_KIND_MDCT1D:
        if ((len & 3) || len == 0) return chfft::set_error(CHFFT_EINVAL_LEN, "invalid length");
        if (p.window == CHFFT_WINDOW_CUSTOM) {
          if (!window_table) return chfft::set_error(CHFFT_EINVAL, "custom window needs a table");
          const auto* w = static_cast<const unsigned char*>(window_table);
          p.custom_window.assign(w, w + len * chfft::real_bytes(p.dtype));
        }
        break;
      default: return chfft::set_error(CHFFT_EINVAL, "setup(len) is not a method of this type");
    }
    p.len = (long long)len;
    return p.build();
  });
}

int chfft_cfft2d_setup(chfft_plan plan, size_t len_m, size_t len_n) {
  if (!plan || plan->impl.kind != CHFFT_KIND_CFFT2D) return chfft::set_error(CHFFT_EINVAL, "not a CFft2D plan");
  PlanImpl& p = plan->impl;
  return guarded([&]() -> int {
    p.len_m = (long long)len_m;
    p.len_n = (long long)len_n;
    p.len = p.len_m * p.len_n;
    return p.build();
  });
}

int chfft_dct1d_setup(chfft_plan plan, int dct_type, size_t len, int is_ortho) {
  if (!plan || plan->impl.kind != CHFFT_KIND_DCT1D) return chfft::set_error(CHFFT_EINVAL, "not a Dct1D plan");
  if (dct_type != CHFFT_DCT_TWO && dct_type != CHFFT_DCT_THREE) return chfft::set_error(CHFFT_EINVAL, "unknown DCT type");
  if ((len & 1) || len == 0) return chfft::set_error(CHFFT_EINVAL_LEN, "invalid length");
  PlanImpl& p = plan->impl;
  return guarded([&]() -> int {
    p.dct_type = dct_type;
    p.len = (long long)len;
    p.ortho = is_ortho != 0;
    return p.build();
  });
}

int chfft_execute(chfft_plan plan, int method, const void* src, size_t src_len, void* dst, size_t dst_len) {
  if (!plan) return chfft::set_error(CHFFT_EINVAL, "null plan");
  PlanImpl& p = plan->impl;
  if (p.kind == CHFFT_KIND_CFFT2D) return chfft::set_error(CHFFT_EINVAL, "use chfft_execute_2d for CFft2D");
  chfft::MethodSpec ms = chfft::method_spec(p.kind, method);
  if (!ms.ok) return chfft::set_error(CHFFT_EINVAL, "method not offered by this type");
  return guarded([&]() -> int {
    if (p.kind == CHFFT_KIND_CFFT1D && (long long)src_len != p.len) {
      // CFft1D re-plans on a new length (src/cfft1d.rs:216-218).
      p.len = (long long)src_len;
      int rc = p.build();
      if (rc != CHFFT_OK) return rc;
    }
    if (src_len != p.in_elems(ms.back) || dst_len != p.out_elems(ms.back)) {
      return chfft::set_error(CHFFT_EINVAL_LEN, "invalid length (source: " + std::to_string(src_len) +
                                                    ", plan: " + std::to_string(p.len) + ")");
    }
    if ((src_len && !src) || (dst_len && !dst)) return chfft::set_error(CHFFT_EINVAL, "null buffer");
    p.exec_host(ms, src, dst, 1);
    return CHFFT_OK;
  });
}

int chfft_execute_2d(chfft_plan plan, int method, const void* src, size_t len_m, size_t len_n, void* dst) {
  if (!plan || plan->impl.kind != CHFFT_KIND_CFFT2D) return chfft::set_error(CHFFT_EINVAL, "not a CFft2D plan");
  PlanImpl& p = plan->impl;
  chfft::MethodSpec ms = chfft::method_spec(p.kind, method);
  if (!ms.ok) return chfft::set_error(CHFFT_EINVAL, "method not offered by CFft2D");
  return guarded([&]() -> int {
    if (len_m == 0 || len_n == 0) return (int)CHFFT_OK;  // empty input -> empty output (src/cfft2d.rs:333-335)
    if ((long long)len_m != p.len_m || (long long)len_n != p.len_n) {  // src/cfft2d.rs:336-338
      p.len_m = (long long)len_m;
      p.len_n = (long long)len_n;
      p.len = p.len_m * p.len_n;
      int rc = p.build();
      if (rc != CHFFT_OK) return rc;
    }
    if (!src || !dst) return chfft::set_error(CHFFT_EINVAL, "null buffer");
    p.exec_host(ms, src, dst, 1);
    return (int)CHFFT_OK;
  });
}

int chfft_execute_batch(chfft_plan plan, int method, const void* src, void* dst, size_t batch) {
  if (!plan) return chfft::set_error(CHFFT_EINVAL, "null plan");
  PlanImpl& p = plan->impl;
  chfft::MethodSpec ms = chfft::method_spec(p.kind, method);
  if (!ms.ok) return chfft::set_error(CHFFT_EINVAL, "method not offered by this type");
  if (batch && (!src || !dst)) return chfft::set_error(CHFFT_EINVAL, "null buffer");
  return guarded([&]() -> int {
    p.exec_host(ms, src, dst, (long long)batch);
    return (int)CHFFT_OK;
  });
}

int chfft_execute_device(chfft_plan plan, int method, const void* d_src, void* d_dst, size_t batch, void* stream) {
  if (!plan) return chfft::set_error(CHFFT_EINVAL, "null plan");
  PlanImpl& p = plan->impl;
  chfft::MethodSpec ms = chfft::method_spec(p.kind, method);
  if (!ms.ok) return chfft::set_error(CHFFT_EINVAL, "method not offered by this type");
  if (batch && (!d_src || !d_dst)) return chfft::set_error(CHFFT_EINVAL, "null buffer");
  return guarded([&]() -> int {
    p.exec(ms, d_src, d_dst, (long long)batch, static_cast<cudaStream_t>(stream));
    return (int)CHFFT_OK;
  });
}

int chfft_plan_get_info(chfft_plan plan, chfft_plan_info* info) {
  if (!plan || !info) return chfft::set_error(CHFFT_EINVAL, "null argument");
  const PlanImpl& p = plan->impl;
  std::memset(info, 0, sizeof(*info));
  info->kind = p.kind;
  info->dtype = p.dtype;
  info->len = (size_t)p.len;
  info->len_m = (size_t)p.len_m;
  info->len_n = (size_t)p.len_n;
  info->fft_len = (size_t)(p.use_big ? p.big.n : p.core.n);
  info->algorithm = p.use_big ? (p.big.blue ? 3 : 2) : (p.core.blue ? 1 : 0);
  info->padded_len = p.use_big ? (p.big.blue ? (size_t)p.big.m : 0) : (p.core.blue ? (size_t)p.core.st.n : 0);
  int k = 0;
  if (p.core.st.npass >= 2) {
    info->radix[k++] = p.core.st.rf;
    for (int i = 0; i < chfft::kNumRadix; i++)
      for (int c = 0; c < p.core.st.mid[i] && k < 24; c++) info->radix[k++] = chfft::radix_at(i);
    if (k < 24) info->radix[k++] = p.core.st.rl;
  } else {
    for (int i = 0; i < chfft::kNumRadix; i++)
      for (int c = 0; c < p.core.st.all[i] && k < 24; c++) info->radix[k++] = chfft::radix_at(i);
  }
  info->npass = k;
  if (p.core.n > 0) {
    chfft::Geo g = chfft::row_geo(p.core, 1 << 20);
    info->seq_per_cta = g.tpb;
    info->threads_per_cta = g.threads;
    info->smem_per_cta = g.smem;
  }
  info->in_elems = p.in_elems(false);
  info->out_elems = p.out_elems(false);
  info->device_bytes = p.core.device_bytes() + p.core2.device_bytes() + p.big.device_bytes() + p.work.bytes +
                       p.aux0.bytes + p.aux1.bytes;
  return CHFFT_OK;
}

// ---- index arithmetic ------------------------------------------------------

// prime_factorization (src/prime_factorization.rs:66-113): divisors are tried
// as 4, then 2, then odd numbers from 3; 4s are emitted when the first odd
// factor (or the end) is reached, and any prime above max_prime empties the list.
int chfft_factorize(size_t len, size_t max_prime, size_t* values, size_t* counts, size_t cap) {
  if (len == 0) return chfft::set_error(-CHFFT_EINVAL, "length 0 has no factorisation");
  std::vector<std::pair<size_t, size_t>> f;
  size_t v = len, cur = 0, cnt = 0, fours = 0;
  auto emit = [&](size_t p) {
    if (p == cur) {
      cnt++;
      return;
    }
    if (cnt > 0) {
      if (cur == 4) {
        fours = cnt;
      } else {
        if (cur > 4 && fours) {
          f.push_back({4, fours});
          fours = 0;
        }
        f.push_back({cur, cnt});
      }
    }
    cur = p;
    cnt = 1;
  };
  bool too_big = false;
  while (v % 4 == 0 && !too_big) {
    v /= 4;
    if (4 > max_prime) too_big = true;
    emit(4);
  }
  if (!too_big && v % 2 == 0) {
    v /= 2;
    if (2 > max_prime) too_big = true;
    emit(2);
  }
  for (size_t d = 3; !too_big && v > 1;) {
    if (v >= d * d) {
      if (v % d == 0) {
        v /= d;
        if (d > max_prime) too_big = true;
        emit(d);
      } else {
        d += 2;
      }
    } else {
      if (v > max_prime) too_big = true;
      emit(v);
      v = 1;
    }
  }
  if (too_big) return 0;
  if (cnt > 0) f.push_back({cur, cnt});
  if (fours) f.push_back({4, fours});
  for (size_t i = 0; i < f.size() && i < cap; i++) {
    values[i] = f[i].first;
    counts[i] = f[i].second;
  }
  return (int)f.size();
}

// calc_bitreverse (src/precompute_utils.rs:70-91): the gather list grows one
// digit at a time; existing entries are scaled by the radix and the new
// digit values appended.
int chfft_digit_reversal(const size_t* values, const size_t* counts, size_t nfactors, size_t* out, size_t out_cap) {
  std::vector<size_t> ids{0};
  for (size_t f = 0; f < nfactors; f++) {
    for (size_t c = 0; c < counts[f]; c++) {
      const size_t r = values[f], l = ids.size();
      for (size_t j = 0; j < l; j++) ids[j] *= r;
      for (size_t i = 1; i < r; i++)
        for (size_t j = 0; j < l; j++) ids.push_back(ids[j] + i);
    }
  }
  if (ids.size() > out_cap) return chfft::set_error(CHFFT_EINVAL_LEN, "output buffer too small");
  std::memcpy(out, ids.data(), ids.size() * sizeof(size_t));
  return CHFFT_OK;
}

// calc_bitreverse2inplace (src/precompute_utils.rs:93-104): for each i the
// position currently holding gather[i] (tracked with an inverse map) is
// swapped into place and recorded.
int chfft_swap_list(const size_t* gather, size_t n, size_t* out) {
  std::vector<size_t> at(n), where(n);
  for (size_t i = 0; i < n; i++) at[i] = where[i] = i;
  for (size_t i = 0; i < n; i++) {
    if (gather[i] >= n) return chfft::set_error(CHFFT_EINVAL, "gather list is not a permutation");
    const size_t r = where[gather[i]];
    if (r < i) return chfft::set_error(CHFFT_EINVAL, "gather list is not a permutation");
    const size_t a = at[i], b = at[r];
    at[i] = b;
    at[r] = a;
    where[b] = i;
    where[a] = r;
    out[i] = r;
  }
  return CHFFT_OK;
}

int chfft_chirp_index_device(size_t len, uint64_t* d_out, void* stream) {
  if (len && !d_out) return chfft::set_error(CHFFT_EINVAL, "null buffer");
  return guarded([&]() -> int {
    CHFFT_CUDA(chfft::gen_table<double>(chfft::Table::CHIRP_INDEX, (long long)len, (long long)len, 0, d_out,
                                        static_cast<cudaStream_t>(stream)));
    return (int)CHFFT_OK;
  });
}

const char* chfft_last_error(void) { return chfft::tl_error.c_str(); }

const char* chfft_status_string(int status) {
  switch (status) {
    case CHFFT_OK: return "ok";
    case CHFFT_EINVAL_LEN: return "invalid length";
    case CHFFT_EINVAL: return "invalid argument";
    case CHFFT_EUNSUPPORTED: return "unsupported size";
    case CHFFT_ECUDA: return "CUDA error";
    case CHFFT_ENOMEM: return "out of device memory";
    case CHFFT_ETIMEOUT: return "device wait timed out";
    default: return "unknown status";
  }
}

const char* chfft_version(void) { return "chfft_gb300 0.1.0 (sm_103a)"; }

int chfft_plan_compiler_available(void) {
  std::string why;
  if (chfft::jit_available(&why)) return 1;
  chfft::tl_error = why;
  return 0;
}

size_t chfft_plan_compiler_cache_size(void) { return chfft::jit_cache_size(); }

}  // extern "C"

namespace chfft {

// Sets the message chfft_last_error returns on this thread (noalloc.cu).
int record_error(int code, const std::string& msg) { return set_error(code, msg); }

// For the no-allocation entry point (noalloc.cu): the four-step core of a
// CFft1D plan and the direction / scale of `method`. Returns a status and
// sets the last error when the plan does not run on the four-step path.
int plan_four_step(chfft_plan plan, int method, const BigCore** big, bool* back, double* scale) {
  if (!plan) return set_error(CHFFT_EINVAL, "null plan");
  const PlanImpl& p = plan->impl;
  if (p.kind != CHFFT_KIND_CFFT1D || !p.use_big)
    return set_error(CHFFT_EINVAL, "the no-allocation entry point runs CFft1D plans on the four-step path only");
  MethodSpec ms = method_spec(p.kind, method);
  if (!ms.ok) return set_error(CHFFT_EINVAL, "method not offered by this type");
  *big = &p.big;
  *back = ms.back;
  *scale = p.scale_value(ms.scale);
  return CHFFT_OK;
}

}  // namespace chfft
