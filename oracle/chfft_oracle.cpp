// C entry points of the CPU oracle (test infrastructure only; see
// chfft_oracle.hpp). Loaded by tests/ and by bench.py's cpu_baseline leg
// through ctypes. Batched calls split the batch over `nthreads` std::threads,
// one plan object per thread, which is how chfft is used concurrently: its
// plans take `&mut self` and are not shared between threads. Every batched
// call reports the wall time of the execution phase alone (plans are built
// before a start barrier), in *exec_seconds when that pointer is non-null.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <memory>
#include <thread>

#include "chfft_oracle.hpp"

using namespace chfft_oracle;

namespace {

using Clock = std::chrono::steady_clock;

// Splits [0, batch) into contiguous chunks, one thread each. Each thread
// builds its plan with make(), waits at a start barrier, then runs
// exec(plan, i) for its items. Returns the execution wall time.
template <class Make, class Exec>
double run_batched(size_t batch, int nthreads, Make make, Exec exec) {
  size_t nt = std::max<size_t>(1, std::min<size_t>((size_t)std::max(nthreads, 1), std::max<size_t>(batch, 1)));
  size_t per = (batch + nt - 1) / nt;
  std::atomic<size_t> ready{0};
  std::vector<Clock::time_point> t0(nt), t1(nt);
  auto body = [&](size_t t) {
    auto plan = make();
    ready.fetch_add(1);
    while (ready.load() < nt) std::this_thread::yield();
    t0[t] = Clock::now();
    size_t a = t * per, b = std::min(batch, a + per);
    for (size_t i = a; i < b; i++) exec(*plan, i);
    t1[t] = Clock::now();
  };
  if (nt == 1) {
    body(0);
  } else {
    std::vector<std::thread> th;
    for (size_t t = 0; t < nt; t++) th.emplace_back(body, t);
    for (auto& x : th) x.join();
  }
  auto start = *std::min_element(t0.begin(), t0.end());
  auto end = *std::max_element(t1.begin(), t1.end());
  return std::chrono::duration<double>(end - start).count();
}

void put(double* p, double v) {
  if (p) *p = v;
}

template <typename T>
int cfft1d_impl(size_t len, int method, const void* in, void* out, size_t batch, int nthreads, double* secs) {
  if (method < 0 || method > 11) return 2;
  auto* src = static_cast<const Cplx<T>*>(in);
  auto* dst = static_cast<Cplx<T>*>(out);
  put(secs, run_batched(
                batch, nthreads, [&] { return std::make_unique<CFft1D<T>>(len ? len : 1); },
                [&](CFft1D<T>& p, size_t i) { p.exec((Method)method, src + i * len, dst + i * len, len); }));
  return 0;
}

// CFft2D methods (src/cfft2d.rs:175-291): no backwardn, no in-place forms.
template <typename T>
int cfft2d_impl(size_t m, size_t n, int method, const void* in, void* out, size_t batch, int nthreads,
                double* secs) {
  T sn = T(1) / T(m * n);
  T su = T(1) / tsqrt<T>(T(m * n));
  bool back;
  T sc;
  switch (method) {
    case FORWARD: case FORWARD0: back = false; sc = T(1); break;
    case FORWARDU: back = false; sc = su; break;
    case FORWARDN: back = false; sc = sn; break;
    case BACKWARD: back = true; sc = sn; break;
    case BACKWARD0: back = true; sc = T(1); break;
    case BACKWARDU: back = true; sc = su; break;
    default: return 2;
  }
  auto* src = static_cast<const Cplx<T>*>(in);
  auto* dst = static_cast<Cplx<T>*>(out);
  put(secs, run_batched(
                batch, nthreads, [&] { return std::make_unique<CFft2D<T>>(m, n); },
                [&](CFft2D<T>& p, size_t i) { p.convert(src + i * m * n, dst + i * m * n, m, n, back, sc); }));
  return 0;
}

// RFft1D methods (src/rfft1d.rs:189-313). Forward: N reals -> N/2+1 complex.
template <typename T>
int rfft1d_impl(size_t len, int method, const void* in, void* out, size_t batch, int nthreads, double* secs) {
  if (len & 1) return 1;
  if (method > BACKWARDN) return 2;
  size_t h = len / 2 + 1;
  put(secs, run_batched(
                batch, nthreads, [&] { return std::make_unique<RFft1D<T>>(len); },
                [&](RFft1D<T>& p, size_t i) {
                  if (method <= FORWARDN) {
                    T sc = method == FORWARDU ? p.scaler_u() : method == FORWARDN ? p.scaler_n() : T(1);
                    p.forward(static_cast<const T*>(in) + i * len, static_cast<Cplx<T>*>(out) + i * h, sc);
                  } else {
                    T sc = (method == BACKWARD || method == BACKWARDN) ? p.scaler_n()
                           : method == BACKWARDU                        ? p.scaler_u()
                                                                        : T(1);
                    p.backward(static_cast<const Cplx<T>*>(in) + i * h, static_cast<T*>(out) + i * len, sc);
                  }
                }));
  return 0;
}

// Dct1D methods (src/dct1d.rs:94-144): forward/forward0 x1, forwardu x s,
// forwardn x s^2 with s = sqrt(2/N).
template <typename T>
int dct1d_impl(int type, size_t len, int ortho, int method, const void* in, void* out, size_t batch, int nthreads,
               double* secs) {
  if (len & 1) return 1;
  if (method > FORWARDN) return 2;
  put(secs, run_batched(
                batch, nthreads, [&] { return std::make_unique<Dct1D<T>>(type, len, ortho != 0); },
                [&](Dct1D<T>& p, size_t i) {
                  T s = p.unitary_scaler();
                  T sc = method == FORWARDU ? s : method == FORWARDN ? s * s : T(1);
                  p.convert(static_cast<const T*>(in) + i * len, static_cast<T*>(out) + i * len, sc);
                }));
  return 0;
}

// Mdct1D methods (src/mdct1d.rs:130-195): forward x sqrt(N/2), forwardu x1,
// backward x 1/sqrt(N/2), backwardu x1. window_kind 0 sine, 1 vorbis,
// 2 custom table of len values.
template <typename T>
int mdct1d_impl(size_t len, int window_kind, const void* window, int method, const void* in, void* out,
                size_t batch, int nthreads, double* secs) {
  if (len & 3) return 1;
  if (method != FORWARD && method != FORWARDU && method != BACKWARD && method != BACKWARDU) return 2;
  std::vector<T> win(len);
  for (size_t i = 0; i < len; i++)
    win[i] = window_kind == 0   ? sine_window<T>(len, i)
             : window_kind == 1 ? vorbis_window<T>(len, i)
                                : static_cast<const T*>(window)[i];
  size_t h = len / 2;
  put(secs, run_batched(
                batch, nthreads, [&] { return std::make_unique<Mdct1D<T>>(win.data(), len); },
                [&](Mdct1D<T>& p, size_t i) {
                  const T* s = static_cast<const T*>(in);
                  T* d = static_cast<T*>(out);
                  switch (method) {
                    case FORWARD: p.forward(s + i * len, d + i * h, p.scaler_ui()); break;
                    case FORWARDU: p.forward(s + i * len, d + i * h, T(1)); break;
                    case BACKWARD: p.backward(s + i * h, d + i * len, p.scaler_u()); break;
                    default: p.backward(s + i * h, d + i * len, T(1)); break;
                  }
                }));
  return 0;
}

}  // namespace

extern "C" {

// Factor list of `len` with primes <= max; returns the number of factors.
int orc_factorize(size_t len, size_t max, size_t* values, size_t* counts, size_t cap) {
  std::vector<Factor> f = prime_factorization(len, max);
  for (size_t i = 0; i < f.size() && i < cap; i++) {
    values[i] = f[i].value;
    counts[i] = f[i].count;
  }
  return (int)f.size();
}

// Digit-reversal gather list for an explicit factor list; `out` holds the
// product of value^count entries.
void orc_bitreverse(size_t len, const size_t* values, const size_t* counts, size_t nf, size_t* out) {
  std::vector<Factor> f;
  for (size_t i = 0; i < nf; i++) f.push_back({values[i], counts[i]});
  std::vector<size_t> ids = calc_bitreverse(len, f);
  std::memcpy(out, ids.data(), ids.size() * sizeof(size_t));
}

void orc_bitreverse2inplace(const size_t* src, size_t n, size_t* out, int literal) {
  std::vector<size_t> s(src, src + n);
  std::vector<size_t> r = literal ? calc_bitreverse2inplace_literal(s) : calc_bitreverse2inplace(s);
  std::memcpy(out, r.data(), n * sizeof(size_t));
}

// Chirp-Z table indices (i*i) % 2N for i < N (src/cfft1d.rs:123-128).
void orc_chirp_index(size_t len, size_t* out) {
  size_t dlen = len << 1;
  for (size_t i = 0; i < len; i++) out[i] = (i * i) % dlen;
}

void orc_omega(int dtype, size_t len, void* out) {
  if (dtype == 0) {
    auto o = calc_omega<float>(len);
    std::memcpy(out, o.data(), o.size() * sizeof(o[0]));
  } else {
    auto o = calc_omega<double>(len);
    std::memcpy(out, o.data(), o.size() * sizeof(o[0]));
  }
}

// 0 = mixed radix, 1 = Chirp-Z; M (the padded power of two) in *pow2len.
int orc_cfft1d_mode(size_t len, size_t* pow2len) {
  std::vector<Factor> f = prime_factorization(len, 7);
  *pow2len = f.empty() ? (next_pow2(len) << 1) : 0;
  return f.empty() ? 1 : 0;
}

int orc_cfft1d(int dtype, size_t len, int method, const void* in, void* out, size_t batch, int nthreads,
               double* secs) {
  return dtype == 0 ? cfft1d_impl<float>(len, method, in, out, batch, nthreads, secs)
                    : cfft1d_impl<double>(len, method, in, out, batch, nthreads, secs);
}

int orc_cfft2d(int dtype, size_t m, size_t n, int method, const void* in, void* out, size_t batch, int nthreads,
               double* secs) {
  return dtype == 0 ? cfft2d_impl<float>(m, n, method, in, out, batch, nthreads, secs)
                    : cfft2d_impl<double>(m, n, method, in, out, batch, nthreads, secs);
}

int orc_rfft1d(int dtype, size_t len, int method, const void* in, void* out, size_t batch, int nthreads,
               double* secs) {
  return dtype == 0 ? rfft1d_impl<float>(len, method, in, out, batch, nthreads, secs)
                    : rfft1d_impl<double>(len, method, in, out, batch, nthreads, secs);
}

int orc_dct1d(int dtype, int type, size_t len, int ortho, int method, const void* in, void* out, size_t batch,
              int nthreads, double* secs) {
  return dtype == 0 ? dct1d_impl<float>(type, len, ortho, method, in, out, batch, nthreads, secs)
                    : dct1d_impl<double>(type, len, ortho, method, in, out, batch, nthreads, secs);
}

int orc_mdct1d(int dtype, size_t len, int window_kind, const void* window, int method, const void* in, void* out,
               size_t batch, int nthreads, double* secs) {
  return dtype == 0 ? mdct1d_impl<float>(len, window_kind, window, method, in, out, batch, nthreads, secs)
                    : mdct1d_impl<double>(len, window_kind, window, method, in, out, batch, nthreads, secs);
}

}  // extern "C"
