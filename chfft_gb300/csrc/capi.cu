// The C ABI (include/chfft_gpu.h): plan objects mirroring chfft's five plan
// types, their setup methods and the per-method (direction, scale) table.
#include <functional>
#include <new>

#include "plan_impl.hpp"

using chfft::Fail;
using chfft::PlanImpl;

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

int chfft_cfft3d_create(int dtype, size_t len_l, size_t len_m, size_t len_n, chfft_plan* out) {
  if (!valid_dtype(dtype)) return chfft::set_error(CHFFT_EINVAL, "unknown dtype");
  if (len_l > (1u << 31) || len_m > (1u << 31) || len_n > (1u << 31)) return chfft::set_error(CHFFT_EINVAL_LEN, "invalid length");
  return create(out, [&](PlanImpl& p) -> int {
    p.kind = CHFFT_KIND_CFFT3D;
    p.dtype = dtype;
    p.len_l = (long long)len_l;
    p.len_m = (long long)len_m;
    p.len_n = (long long)len_n;
    p.len = p.len_l * p.len_m * p.len_n;
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
  if (p.kind == CHFFT_KIND_CFFT3D) return chfft::set_error(CHFFT_EINVAL, "use chfft_execute_3d for CFft3D");
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

int chfft_execute_3d(chfft_plan plan, int method, const void* src, size_t len_l, size_t len_m, size_t len_n,
                     void* dst) {
  if (!plan || plan->impl.kind != CHFFT_KIND_CFFT3D) return chfft::set_error(CHFFT_EINVAL, "not a CFft3D plan");
  PlanImpl& p = plan->impl;
  chfft::MethodSpec ms = chfft::method_spec(p.kind, method);
  if (!ms.ok) return chfft::set_error(CHFFT_EINVAL, "method not offered by CFft3D");
  return guarded([&]() -> int {
    if (len_l == 0 || len_m == 0 || len_n == 0) return (int)CHFFT_OK;  // empty in, empty out (as CFft2D)
    if ((long long)len_l != p.len_l || (long long)len_m != p.len_m || (long long)len_n != p.len_n) {
      p.len_l = (long long)len_l;
      p.len_m = (long long)len_m;
      p.len_n = (long long)len_n;
      p.len = p.len_l * p.len_m * p.len_n;
      int rc = p.build();
      if (rc != CHFFT_OK) return rc;
    }
    if (!src || !dst) return chfft::set_error(CHFFT_EINVAL, "null buffer");
    p.exec_host(ms, src, dst, 1);
    return (int)CHFFT_OK;
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

int chfft_execute_device_split(chfft_plan plan, int method, const void* d_src_re, const void* d_src_im,
                               void* d_dst_re, void* d_dst_im, size_t batch, void* stream) {
  if (!plan) return chfft::set_error(CHFFT_EINVAL, "null plan");
  PlanImpl& p = plan->impl;
  chfft::MethodSpec ms = chfft::method_spec(p.kind, method);
  if (!ms.ok) return chfft::set_error(CHFFT_EINVAL, "method not offered by this type");
  if (batch && (!d_src_re || !d_src_im || !d_dst_re || !d_dst_im)) return chfft::set_error(CHFFT_EINVAL, "null buffer");
  return guarded([&]() -> int {
    p.exec_split(ms, d_src_re, d_src_im, d_dst_re, d_dst_im, (long long)batch, static_cast<cudaStream_t>(stream));
    return (int)CHFFT_OK;
  });
}

int chfft_execute_device_strided(chfft_plan plan, int method, const void* d_src, size_t istride, size_t idist,
                                 void* d_dst, size_t ostride, size_t odist, size_t batch, void* stream) {
  if (!plan) return chfft::set_error(CHFFT_EINVAL, "null plan");
  PlanImpl& p = plan->impl;
  chfft::MethodSpec ms = chfft::method_spec(p.kind, method);
  if (!ms.ok) return chfft::set_error(CHFFT_EINVAL, "method not offered by this type");
  if (batch && (!d_src || !d_dst)) return chfft::set_error(CHFFT_EINVAL, "null buffer");
  return guarded([&]() -> int {
    p.exec_strided(ms, d_src, (long long)istride, (long long)idist, d_dst, (long long)ostride, (long long)odist,
                   (long long)batch, static_cast<cudaStream_t>(stream));
    return (int)CHFFT_OK;
  });
}

int chfft_plan_wait(chfft_plan plan, void* stream) {
  if (!plan) return chfft::set_error(CHFFT_EINVAL, "null plan");
  PlanImpl& p = plan->impl;
  return guarded([&]() -> int {
    CHFFT_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
    p.check_waits();
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
  info->len_l = (size_t)p.len_l;
  info->len_n = (size_t)p.len_n;
  info->fft_len = (size_t)(p.use_big ? p.big.n : p.use_rader ? p.rader.n : p.core.n);
  info->algorithm = p.use_big ? (p.big.blue ? 3 : 2) : p.use_rader ? 4 : (p.core.blue ? 1 : 0);
  info->padded_len = p.use_big ? (p.big.blue ? (size_t)p.big.m : 0)
                               : p.use_rader ? 0 : (p.core.blue ? (size_t)p.core.st.n : 0);
  // Rader plans report their (n - 1)-point core's passes and geometry.
  const chfft::Core& cc = p.use_rader ? p.rader.lc : p.core;
  int k = 0;
  if (cc.st.npass >= 2) {
    info->radix[k++] = cc.st.rf;
    for (int i = 0; i < chfft::kNumRadix; i++)
      for (int c = 0; c < cc.st.mid[i] && k < 24; c++) info->radix[k++] = chfft::radix_at(i);
    if (k < 24) info->radix[k++] = cc.st.rl;
  } else {
    for (int i = 0; i < chfft::kNumRadix; i++)
      for (int c = 0; c < cc.st.all[i] && k < 24; c++) info->radix[k++] = chfft::radix_at(i);
  }
  info->npass = k;
  if (cc.n > 0) {
    int ldr = 0;
    chfft::Geo g = p.use_rader ? chfft::rader_geo(p.rader, 1 << 20, p.opts, &ldr) : chfft::row_geo(p.core, 1 << 20);
    info->seq_per_cta = g.tpb;
    info->threads_per_cta = g.threads;
    info->smem_per_cta = g.smem;
  }
  info->in_elems = p.in_elems(false);
  info->out_elems = p.out_elems(false);
  info->device_bytes = p.core.device_bytes() + p.core2.device_bytes() + p.core3.device_bytes() + p.big.device_bytes() + p.work.bytes +
                       p.aux0.bytes + p.aux1.bytes + p.rader.device_bytes() + p.clus.device_bytes();
  info->cluster_ctas = p.clus.n ? p.clus.csize : 0;
  info->cluster_n1 = p.clus.n ? (size_t)p.clus.n1 : 0;
  info->cluster_n2 = p.clus.n ? (size_t)p.clus.n2 : 0;
  info->cluster_max_batch = p.clus.n ? (size_t)p.clus.max_batch : 0;
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

// Sets / clears the message chfft_last_error returns on this thread (noalloc.cu).
int record_error(int code, const std::string& msg) { return set_error(code, msg); }
void clear_error() { tl_error.clear(); }

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
