// Plan tuning: the knobs' search space, the cost-model features of a
// configuration, the exhaustive autotuner and the learned proposal. There is
// no reference counterpart: chfft derives one plan per length from its fixed
// factor order (src/prime_factorization.rs:66-113) and its Chirp-Z length
// rule (src/cfft1d.rs:114-140).
#include <algorithm>
#include <cmath>
#include <string>
#include <tuple>
#include <vector>

#include "plan_impl.hpp"

namespace chfft {

int record_error(int code, const std::string& msg);

namespace {

PlanOpts to_opts(const chfft_plan_config& c) {
  PlanOpts o;
  o.k1 = c.k1;
  o.tpb = c.seq_per_cta;
  o.max_radix = c.max_radix;
  o.jit = c.jit;
  o.blue_m = c.bluestein_len;
  o.fs_n1 = c.fs_n1;
  o.fs_tpb = c.tile_cols;
  o.l2_mb = c.l2_chunk_mb;
  o.tc = c.tc_precision;
  o.min_blocks = c.min_blocks_per_sm;
  o.balance = c.balanced;
  o.ept = c.col_elems_per_thread;
  return o;
}

chfft_plan_config to_cfg(const PlanOpts& o) {
  chfft_plan_config c;
  c.k1 = o.k1;
  c.seq_per_cta = o.tpb;
  c.max_radix = o.max_radix;
  c.jit = o.jit;
  c.bluestein_len = o.blue_m;
  c.fs_n1 = o.fs_n1;
  c.tile_cols = o.fs_tpb;
  c.l2_chunk_mb = o.l2_mb;
  c.tc_precision = o.tc;
  c.min_blocks_per_sm = o.min_blocks;
  c.balanced = o.balance;
  c.l2_prefetch = 0;     // retired knobs: always reported off
  c.l2_evict_hints = 0;
  c.col_elems_per_thread = o.ept;
  return c;
}

double lg2(double v) { return v > 0 ? std::log2(v) : 0.0; }

bool jit_on() {
  static int ok = -1;
  if (ok < 0) ok = jit_available(nullptr) ? 1 : 0;
  return ok == 1;
}

// A Core carrying only a stage list (geometry queries, no device tables).
Core shell(const StageList& st, int dtype) {
  Core c;
  c.st = st;
  c.sw = st;
  c.n = st.n;
  c.dtype = dtype;
  return c;
}

// The launch structure (plan, batch, knobs) resolves to, derived on the host
// from the knobs alone: features and de-duplication use it.
struct Resolved {
  bool big = false, blue = false, k1 = false, jit = false, wide = false;
  int tpb = 1, threads = 0, tile = 0, n1 = 0, n2 = 0;
  size_t smem = 0;
  long long fft_len = 0, ctas = 0, chunks = 1, l2mb = 0;
  int cnt[kNumRadix] = {0};
  int npass = 0, rfirst = 0, rlast = 0;
  int minb = 0;          // specialised kernels: launch-bounds CTAs per SM
  bool balanced = false;  // specialised kernels: balanced mixed-radix variant
  int prefetch = 0;       // retired next-wave L2 prefetch knob: always 0 (feature slot kept)

  auto key() const {
    return std::make_tuple(big, blue, k1, jit, wide, tpb, tile, n1, fft_len, l2mb, chunks, minb, balanced, prefetch);
  }
};

void add_stages(Resolved& r, const StageList& st) {
  for (int i = 0; i < kNumRadix; i++) r.cnt[i] += st.all[i];
  r.npass += st.npass;
  const std::vector<int> ord = pass_order(st);
  if (!ord.empty()) {
    if (!r.rfirst) r.rfirst = ord.front();
    r.rlast = ord.back();
  }
}

// Stage list the specialised kernel runs for this geometry (radix 32 when allowed).
StageList effective(const StageList& st, int dtype, const Geo& g, bool jit, bool* wide) {
  *wide = false;
  if (!jit || g.k1 || g.max_radix < 32 || dtype != 0 || st.n < 2) return st;
  StageList w;
  if (!make_stages(st.n, &w, 32) || pass_order(w) == pass_order(st)) return st;
  if (threads_needed(w, ept_of(dtype), g.tpb, false) > kMaxThreads) return st;
  *wide = true;
  return w;
}

bool four_step_pair(long long m, int dtype, int want_n1, int* n1, int* n2) {
  if (want_n1 > 1 && m % want_n1 == 0) {
    StageList a, b;
    if (make_stages(want_n1, &a) && make_stages(m / want_n1, &b) && fits_cta(a, dtype) && fits_cta(b, dtype)) {
      *n1 = want_n1;
      *n2 = (int)(m / want_n1);
      return true;
    }
  }
  return four_step_split(m, dtype, n1, n2);
}

Resolved resolve(const PlanImpl& p, long long batch, const PlanOpts& o) {
  Resolved r;
  const int dt = p.dtype;
  auto one_cta = [&](const StageList& st, long long count) {
    const Core c = shell(st, dt);
    const Geo g = row_geo(c, count, o);
    r.jit = jit_on() && want_specialised(count * st.n, o.jit);
    bool wide = false;
    const StageList e = effective(st, dt, g, r.jit, &wide);
    r.wide = wide;
    r.k1 = g.k1;
    r.tpb = g.tpb;
    r.threads = wide ? std::max(32, (threads_needed(e, ept_of(dt), g.tpb, false) + 31) / 32 * 32) : g.threads;
    r.smem = g.smem;
    r.ctas = (count + g.tpb - 1) / g.tpb;
    r.minb = r.jit ? (o.min_blocks > 0 ? o.min_blocks : (g.k1 ? 2 : 1)) : 0;
    if (r.jit && g.k1 && o.balance != 0) {
      int rmin = 1 << 30, rmax = 0;
      for (int x : pass_order(e)) {
        rmin = std::min(rmin, x);
        rmax = std::max(rmax, x);
      }
      bool divides = rmax > 0;
      for (int x : pass_order(e)) divides = divides && rmax % x == 0;
      r.balanced = rmax > rmin && divides;
    }
    add_stages(r, e);
  };
  switch (p.kind) {
    case CHFFT_KIND_CFFT1D: {
      if (p.len <= 1) break;
      if (p.use_big) {
        r.big = true;
        r.blue = p.big.blue;
        const long long m = p.big.m;
        r.fft_len = m;
        four_step_pair(m, dt, o.fs_n1, &r.n1, &r.n2);
        StageList sa, sb;
        make_stages(r.n1, &sa);
        make_stages(r.n2, &sb);
        const Core ca = shell(sa, dt);
        const int tile_default = o.fs_tpb > 0 ? o.fs_tpb : (dt == 0 ? 8 : 0);
        const Geo ga = col_geo(ca, r.n2, tile_default, o);
        r.jit = jit_on() && want_specialised(batch * m, o.jit);
        bool wide = false;
        const StageList ea = effective(sa, dt, ga, r.jit, &wide);
        bool wide_b = false;
        const StageList eb = effective(sb, dt, col_geo(shell(sb, dt), r.n1, tile_default, o), r.jit, &wide_b);
        r.wide = wide || wide_b;
        r.k1 = ga.k1;
        r.tpb = ga.tpb;
        r.tile = ga.tpb;
        r.threads = ga.threads;
        r.smem = ga.smem;
        r.l2mb = o.l2_mb > 0 ? o.l2_mb : 512;
        const long long per = m * (long long)cplx_bytes(dt) * (r.blue ? 2 : 1);
        const long long chunk = std::max(1LL, std::min(batch, (r.l2mb << 20) / per));
        r.chunks = (batch + chunk - 1) / chunk;
        r.ctas = chunk * ((r.n2 + ga.tpb - 1) / ga.tpb);
        add_stages(r, ea);
        add_stages(r, eb);
      } else {
        StageList st = p.core.st;
        r.blue = p.core.blue;
        if (r.blue) {
          long long mm = bluestein_length(p.len, dt);
          StageList sb;
          if (o.blue_m >= 2 * p.len - 1 && make_stages(o.blue_m, &sb) && fits_cta(sb, dt)) mm = o.blue_m;
          make_stages(mm, &st);
        }
        r.fft_len = st.n;
        one_cta(st, batch);
      }
      break;
    }
    case CHFFT_KIND_CFFT2D: {
      if (p.len_m == 0 || p.len_n == 0) break;
      r.fft_len = p.core.st.n;
      one_cta(p.core.st, batch * p.len_m);
      const Geo gc = col_geo(p.core2, (int)p.len_n, o.fs_tpb, o);
      r.tile = gc.tpb;
      r.ctas += batch * ((p.len_n + gc.tpb - 1) / gc.tpb);
      add_stages(r, p.core2.st);
      break;
    }
    default:
      r.fft_len = p.core.st.n;
      r.blue = p.core.blue;
      one_cta(p.core.st, batch);
      break;
  }
  return r;
}

// chfft's own factor list of len (src/prime_factorization.rs:66-113): 4s,
// then a 2, then odd primes; counts of 4, 2, 3, 5, 7 and the largest prime.
void chfft_factors(long long len, int* c4, int* c2, int* c3, int* c5, int* c7, long long* pmax) {
  *c4 = *c2 = *c3 = *c5 = *c7 = 0;
  *pmax = 1;
  long long n = len;
  int twos = 0;
  while (n > 1 && n % 2 == 0) {
    n /= 2;
    twos++;
  }
  if (twos) *pmax = 2;
  *c4 = twos / 2;
  *c2 = twos % 2;
  for (long long d = 3; d * d <= n; d += 2)
    while (n % d == 0) {
      n /= d;
      *pmax = std::max(*pmax, d);
      if (d == 3) (*c3)++;
      if (d == 5) (*c5)++;
      if (d == 7) (*c7)++;
    }
  if (n > 1) {
    *pmax = std::max(*pmax, n);
    if (n == 3) (*c3)++;
    if (n == 5) (*c5)++;
    if (n == 7) (*c7)++;
  }
}

void features(const PlanImpl& p, long long batch, const PlanOpts& o, float* f) {
  const Resolved r = resolve(p, batch, o);
  for (int i = 0; i < CHFFT_FEATURES; i++) f[i] = 0.f;
  const long long len = p.kind == CHFFT_KIND_CFFT2D ? p.len_m * p.len_n : p.len;
  int c4, c2, c3, c5, c7;
  long long pmax;
  chfft_factors(p.kind == CHFFT_KIND_CFFT2D ? p.len_n : len, &c4, &c2, &c3, &c5, &c7, &pmax);
  int k = 0;
  f[k++] = (float)lg2((double)len);
  f[k++] = (float)lg2((double)r.fft_len);
  f[k++] = r.blue ? 1.f : 0.f;
  f[k++] = r.big ? 1.f : 0.f;
  f[k++] = (float)c4;
  f[k++] = (float)c2;
  f[k++] = (float)c3;
  f[k++] = (float)c5;
  f[k++] = (float)c7;
  f[k++] = (float)lg2((double)pmax);
  f[k++] = (float)lg2((double)batch);
  f[k++] = (float)p.dtype;
  f[k++] = (float)p.kind;
  f[k++] = r.balanced ? 0.5f : (r.k1 ? 1.f : 0.f);
  f[k++] = (float)lg2((double)r.tpb);
  f[k++] = (float)r.threads / kMaxThreads;
  f[k++] = (float)r.smem / (float)kMaxSmem;
  f[k++] = (float)lg2((double)std::max(1LL, r.ctas));
  f[k++] = r.jit ? 1.f : 0.f;
  f[k++] = r.wide ? 1.f : 0.f;
  f[k++] = (float)r.npass;
  for (int i = 0; i < kNumRadix; i++) f[k++] = (float)r.cnt[i];  // stage multiset (16 8 4 2 10 5 3 7 32)
  f[k++] = (float)r.rfirst / 32.f;
  f[k++] = (float)r.rlast / 32.f;
  f[k++] = r.blue ? (float)lg2((double)r.fft_len / (double)len) : 0.f;
  f[k++] = (float)lg2((double)r.n1);
  f[k++] = (float)lg2((double)r.n2);
  f[k++] = (float)lg2((double)r.tile);
  f[k++] = (float)lg2((double)r.l2mb);
  f[k++] = (float)lg2((double)len * (double)batch);
  f[k++] = (float)lg2((double)r.chunks);
  f[k++] = (float)r.minb;
  f[k++] = (float)r.prefetch;
}

// Bluestein lengths to try: the cheapest M by the engine's cost rule and the
// next cheapest ones (7-smooth, >= 2n - 1, one CTA).
std::vector<long long> blue_lengths(long long n, int dtype, int count) {
  std::vector<std::pair<double, long long>> c;
  long long lo = 2 * n - 1, hi = 1;
  while (hi < lo) hi <<= 1;
  for (long long m = lo; m <= hi; m++) {
    StageList st;
    if (!make_stages(m, &st) || !fits_cta(st, dtype)) continue;
    c.push_back({(double)m * (st.npass + 0.5), m});
  }
  std::sort(c.begin(), c.end());
  std::vector<long long> out;
  for (size_t i = 0; i < c.size() && (int)out.size() < count; i++) out.push_back(c[i].second);
  return out;
}

// Candidate 0 is always the built-in heuristic (every knob on auto).
std::vector<PlanOpts> candidates(const PlanImpl& p, long long batch, bool tune_jit) {
  std::vector<PlanOpts> raw{PlanOpts{}};
  PlanOpts base;
  std::vector<std::pair<int, int>> jits = {{-1, 0}};
  if (tune_jit) {
    jits = {{0, 0}, {1, 16}};
    if (p.dtype == 0) jits.push_back({1, 32});
  }
  const int dt = p.dtype;
  auto row_knobs = [&](const StageList& st, long long count, std::vector<PlanOpts>& out, PlanOpts o) {
    const int t1k = threads_needed(st, ept_of(dt), 1, true);
    if (t1k <= kMaxThreads) {
      const int tmax = std::max(1, kMaxThreads / t1k);
      for (int t : {tmax, tmax / 2, tmax / 4, 1}) {
        if (t < 1 || t > count) continue;
        o.k1 = 1;
        o.tpb = t;
        out.push_back(o);
        if (o.jit == 1) {  // a tighter register budget for a third resident CTA; no balancing
          PlanOpts q = o;
          q.min_blocks = 3;
          out.push_back(q);
          q = o;
          q.balance = 0;
          out.push_back(q);
        }
      }
    }
    for (int t : {1, 2, 4, 8}) {
      if (t > count) continue;
      o.k1 = 0;
      o.tpb = t;
      out.push_back(o);
    }
  };
  for (auto [jit, mr] : jits) {
    base.jit = jit;
    base.max_radix = mr;
    switch (p.kind) {
      case CHFFT_KIND_CFFT1D:
        if (p.len <= 1) {
          raw.push_back(base);
        } else if (p.use_big) {
          // Splits: the balanced one and the neighbouring divisors.
          std::vector<std::pair<double, int>> sp;
          const long long m = p.big.m;
          const long long cap = dt == 0 ? 2048 : 1024;
          for (long long d = 2; d <= cap; d++) {
            if (m % d) continue;
            StageList a, b;
            if (!make_stages(d, &a) || !make_stages(m / d, &b) || !fits_cta(a, dt) || !fits_cta(b, dt)) continue;
            sp.push_back({std::fabs(std::log((double)d) - 0.5 * std::log((double)m)), (int)d});
          }
          std::sort(sp.begin(), sp.end());
          for (size_t i = 0; i < sp.size() && i < 3; i++)
            for (int tile : dt == 0 ? std::vector<int>{8, 16} : std::vector<int>{4, 8})
              for (int l2 : {64, 512}) {
                PlanOpts o = base;
                o.fs_n1 = sp[i].second;
                o.fs_tpb = tile;
                o.l2_mb = l2;
                raw.push_back(o);
              }
        } else if (p.core.blue) {
          for (long long mm : blue_lengths(p.len, dt, 3)) {
            PlanOpts o = base;
            o.blue_m = mm;
            StageList st;
            make_stages(mm, &st);
            row_knobs(st, batch, raw, o);
          }
        } else {
          row_knobs(p.core.st, batch, raw, base);
        }
        break;
      case CHFFT_KIND_CFFT2D: {
        if (p.len_m == 0 || p.len_n == 0) {
          raw.push_back(base);
          break;
        }
        std::vector<PlanOpts> rows;
        row_knobs(p.core.st, batch * p.len_m, rows, base);
        for (const PlanOpts& o : rows)
          for (int tile : dt == 0 ? std::vector<int>{4, 8, 16} : std::vector<int>{4, 8}) {
            PlanOpts q = o;
            q.fs_tpb = tile;
            raw.push_back(q);
          }
        break;
      }
      default:
        row_knobs(p.core.st, batch, raw, base);
        break;
    }
  }
  // One config per distinct launch structure.
  std::vector<PlanOpts> out;
  std::vector<decltype(Resolved{}.key())> seen;
  for (const PlanOpts& o : raw) {
    const auto k = resolve(p, batch, o).key();
    if (std::find(seen.begin(), seen.end(), k) != seen.end()) continue;
    seen.push_back(k);
    out.push_back(o);
  }
  if (out.empty()) out.push_back(PlanOpts{});
  return out;
}

template <class F>
int guard(F&& f) {
  try {
    return f();
  } catch (const Fail& e) {
    return record_error(e.code, e.msg);
  } catch (const std::exception& e) {
    return record_error(CHFFT_EINVAL, e.what());
  }
}

}  // namespace
}  // namespace chfft

using chfft::PlanImpl;
using chfft::PlanOpts;

extern "C" {

void chfft_plan_config_default(chfft_plan_config* cfg) {
  if (cfg) *cfg = chfft::to_cfg(PlanOpts{});
}

int chfft_plan_set_config(chfft_plan plan, const chfft_plan_config* cfg) {
  if (!plan || !cfg) return chfft::record_error(CHFFT_EINVAL, "null argument");
  return chfft::guard([&]() -> int {
    plan->impl.apply(chfft::to_opts(*cfg));
    return CHFFT_OK;
  });
}

int chfft_plan_get_config(chfft_plan plan, chfft_plan_config* cfg) {
  if (!plan || !cfg) return chfft::record_error(CHFFT_EINVAL, "null argument");
  *cfg = chfft::to_cfg(plan->impl.opts);
  return CHFFT_OK;
}

int chfft_plan_candidates(chfft_plan plan, size_t batch, int tune_jit, chfft_plan_config* out, int cap, int* n) {
  if (!plan || !n || batch == 0 || (cap > 0 && !out)) return chfft::record_error(CHFFT_EINVAL, "bad argument");
  return chfft::guard([&]() -> int {
    const auto c = chfft::candidates(plan->impl, (long long)batch, tune_jit != 0);
    *n = (int)c.size();
    for (int i = 0; i < cap && i < (int)c.size(); i++) out[i] = chfft::to_cfg(c[i]);
    return CHFFT_OK;
  });
}

int chfft_plan_features(chfft_plan plan, size_t batch, const chfft_plan_config* cfg, float* out) {
  if (!plan || !cfg || !out || batch == 0) return chfft::record_error(CHFFT_EINVAL, "bad argument");
  return chfft::guard([&]() -> int {
    chfft::features(plan->impl, (long long)batch, chfft::to_opts(*cfg), out);
    return CHFFT_OK;
  });
}

int chfft_autotune(chfft_plan plan, int method, size_t batch, int reps, int tune_jit, chfft_plan_config* cfgs,
                   float* ms, int cap, int* n, int* best) {
  if (!plan || batch == 0 || reps < 1 || (cap > 0 && (!cfgs || !ms))) return chfft::record_error(CHFFT_EINVAL, "bad argument");
  return chfft::guard([&]() -> int {
    PlanImpl& p = plan->impl;
    const chfft::MethodSpec spec = chfft::method_spec(p.kind, method);
    if (!spec.ok) return chfft::set_error(CHFFT_EINVAL, "method not offered by this type");
    const auto cands = chfft::candidates(p, (long long)batch, tune_jit != 0);
    cudaStream_t s = p.host_stream();
    const size_t ib = p.in_elems(spec.back) * p.in_esize(spec.back) * batch;
    const size_t ob = p.out_elems(spec.back) * p.out_esize(spec.back) * batch;
    chfft::DevBuf din, dout;
    din.ensure(std::max<size_t>(ib, 16));
    dout.ensure(std::max<size_t>(ob, 16));
    // Finite, normal inputs (every float / double byte 0x3c).
    CHFFT_CUDA(cudaMemsetAsync(din.p, 0x3c, ib, s));
    cudaEvent_t e0, e1;
    CHFFT_CUDA(cudaEventCreate(&e0));
    CHFFT_CUDA(cudaEventCreate(&e1));
    std::vector<float> times(cands.size());
    int ib_best = 0;
    try {
      for (size_t i = 0; i < cands.size(); i++) {
        p.apply(cands[i]);
        p.exec(spec, din.p, dout.p, (long long)batch, s);  // warm-up (and plan-time compile)
        std::vector<float> t(reps);
        for (int r = 0; r < reps; r++) {
          CHFFT_CUDA(cudaEventRecord(e0, s));
          p.exec(spec, din.p, dout.p, (long long)batch, s);
          CHFFT_CUDA(cudaEventRecord(e1, s));
          CHFFT_CUDA(cudaEventSynchronize(e1));
          CHFFT_CUDA(cudaEventElapsedTime(&t[r], e0, e1));
        }
        std::nth_element(t.begin(), t.begin() + reps / 2, t.end());
        times[i] = t[reps / 2];
        if (times[i] < times[ib_best]) ib_best = (int)i;
      }
    } catch (...) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    p.apply(cands[ib_best]);
    if (n) *n = (int)cands.size();
    if (best) *best = ib_best;
    for (int i = 0; i < cap && i < (int)cands.size(); i++) {
      cfgs[i] = chfft::to_cfg(cands[i]);
      ms[i] = times[i];
    }
    return CHFFT_OK;
  });
}

int chfft_plan_propose(chfft_plan plan, size_t batch, chfft_mlp m, int tune_jit, chfft_plan_config* chosen) {
  if (!plan || !m || batch == 0) return chfft::record_error(CHFFT_EINVAL, "bad argument");
  return chfft::guard([&]() -> int {
    PlanImpl& p = plan->impl;
    const auto cands = chfft::candidates(p, (long long)batch, tune_jit != 0);
    std::vector<float> X(cands.size() * CHFFT_FEATURES), y(cands.size());
    for (size_t i = 0; i < cands.size(); i++) chfft::features(p, (long long)batch, cands[i], &X[i * CHFFT_FEATURES]);
    const int rc = chfft_mlp_predict(m, X.data(), (int)cands.size(), y.data());
    if (rc != CHFFT_OK) return rc;
    const size_t b = std::min_element(y.begin(), y.end()) - y.begin();
    p.apply(cands[b]);
    if (chosen) *chosen = chfft::to_cfg(cands[b]);
    return CHFFT_OK;
  });
}

}  // extern "C"
