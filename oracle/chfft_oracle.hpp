// CPU oracle: a C++17 restatement of chfft 0.3.4's transform algorithms.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker that the CUDA path is
// compared against (tests/, __graft_entry__.smoke() and the cpu_baseline leg
// of bench.py). It is never linked into, loaded by or called from the product
// library under chfft_gb300/.
//
// Parity status: the reference is a Rust crate and cannot be built in this
// environment (no cargo/rustc, its num-complex/num-traits dependencies are not
// available offline), so bit-level parity with the Rust binary is UNPINNED.
// The restatement is pinned instead to the reference's own test criteria
// (naive-DFT oracles, round trips and tolerances of src/lib.rs:48-58) and to
// an independent numpy.fft cross-check; see tests/test_oracle.py.
//
// Each function follows the reference operation for operation and cites the
// file:line it restates. Arithmetic follows num-complex 0.4 (Cargo.toml:20;
// third-party, not vendored): complex multiply (ac-bd, ad+bc), `scale` is a
// per-component multiply, `from_polar(r,t)` is (r cos t, r sin t) and `i()`
// is (0,1). Trigonometry uses libm in the working precision T, as num-traits
// 0.2 (Cargo.toml:19) does, so f32 tables are computed in f32 like the
// reference. Build with -ffp-contract=off: rustc does not contract a*b+c.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <vector>

namespace chfft_oracle {

template <typename T>
struct Cplx {
  T re, im;
};

template <typename T> inline Cplx<T> cadd(Cplx<T> a, Cplx<T> b) { return {a.re + b.re, a.im + b.im}; }
template <typename T> inline Cplx<T> csub(Cplx<T> a, Cplx<T> b) { return {a.re - b.re, a.im - b.im}; }
template <typename T> inline Cplx<T> cmul(Cplx<T> a, Cplx<T> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename T> inline Cplx<T> cscale(Cplx<T> a, T s) { return {a.re * s, a.im * s}; }
template <typename T> inline Cplx<T> cconj(Cplx<T> a) { return {a.re, -a.im}; }
template <typename T> inline Cplx<T> cone() { return {T(1), T(0)}; }
template <typename T> inline Cplx<T> czero() { return {T(0), T(0)}; }
// Complex::i() * w with num-complex's multiply: (0*w.re - 1*w.im, 0*w.im + 1*w.re).
template <typename T> inline Cplx<T> cmul_i(Cplx<T> w) { return cmul(Cplx<T>{T(0), T(1)}, w); }
// QuarterRotation (src/lib.rs:27-39): z*i and z*(-i) without a multiply.
template <typename T> inline Cplx<T> quarter_turn(Cplx<T> z) { return {-z.im, z.re}; }
template <typename T> inline Cplx<T> three_quarter_turn(Cplx<T> z) { return {z.im, -z.re}; }

template <typename T> inline T tsin(T x);
template <> inline float tsin<float>(float x) { return sinf(x); }
template <> inline double tsin<double>(double x) { return sin(x); }
template <typename T> inline T tcos(T x);
template <> inline float tcos<float>(float x) { return cosf(x); }
template <> inline double tcos<double>(double x) { return cos(x); }
template <typename T> inline T tsqrt(T x);
template <> inline float tsqrt<float>(float x) { return sqrtf(x); }
template <> inline double tsqrt<double>(double x) { return sqrt(x); }
template <typename T> inline T tpi() { return T(3.14159265358979323846264338327950288); }

inline unsigned tz(size_t v) { return v == 0 ? 64u : (unsigned)__builtin_ctzll((unsigned long long)v); }
inline size_t next_pow2(size_t v) {
  size_t p = 1;
  while (p < v) p <<= 1;
  return p;
}

// ---------------------------------------------------------------- a1 factorizer
struct Factor {
  size_t value, count;
};

// FactorIterator::next (src/prime_factorization.rs:19-60): 4s first, then one
// 2, then odd trial divisors; the last remaining cofactor is emitted as is.
struct FactorIterator {
  size_t value, prime;
  bool next(size_t* out) {
    for (;;) {
      if (prime == 4) {
        if (tz(value) >= 2) {
          value >>= 2;
          *out = 4;
          return true;
        }
        prime = 2;
      } else if (prime == 2) {
        if ((value & 1) == 0) {
          value >>= 1;
          *out = 2;
          return true;
        }
        prime = 3;
      } else {
        if (value >= prime * prime) {
          if (value % prime == 0) {
            value /= prime;
            *out = prime;
            return true;
          }
          prime += 2;
        } else if (value > 1) {
          *out = value;
          value = 0;
          return true;
        } else {
          return false;
        }
      }
    }
  }
};

// prime_factorization (src/prime_factorization.rs:66-113). Returns an empty
// list when any prime factor exceeds `max`. The 4s are held back and emitted
// before the first odd factor (or last), which gives orders such as
// 1000 -> [2^1, 5^3, 4^1]. value 0 loops forever in the reference
// (0 has unbounded trailing zeros); it is rejected here.
inline std::vector<Factor> prime_factorization(size_t value, size_t max) {
  if (value == 0) throw std::invalid_argument("prime_factorization(0) does not terminate in chfft");
  std::vector<Factor> factors;
  size_t count = 0, prime = 0, fac4count = 0;
  FactorIterator it{value, 4};
  size_t p;
  while (it.next(&p)) {
    if (p > max) return {};
    if (prime != p) {
      if (count > 0) {
        if (prime == 4) {
          fac4count = count;
        } else {
          if (prime > 4 && fac4count != 0) {
            factors.push_back({4, fac4count});
            fac4count = 0;
          }
          factors.push_back({prime, count});
        }
      }
      count = 1;
      prime = p;
    } else {
      count += 1;
    }
  }
  if (count > 0) factors.push_back({prime, count});
  if (fac4count != 0) factors.push_back({4, fac4count});
  return factors;
}

// ---------------------------------------------------------------- a2 twiddles
// calc_omega_item (src/precompute_utils.rs:15-21): ((-2*pi)/len)*pos in T.
template <typename T>
inline Cplx<T> calc_omega_item(size_t len, size_t position) {
  T ang = T(-2.0) * tpi<T>() / T(len) * T(position);
  return {T(1) * tcos(ang), T(1) * tsin(ang)};
}

// calc_omega (src/precompute_utils.rs:23-68): len+1 entries, using quarter-
// and half-turn symmetry when 4 | len or 2 | len.
template <typename T>
inline std::vector<Cplx<T>> calc_omega(size_t len) {
  std::vector<Cplx<T>> omega;
  omega.reserve(len + 1);
  omega.push_back(cone<T>());
  if (tz(len) >= 2) {
    size_t q = len >> 2, h = len >> 1;
    for (size_t i = 1; i < q; i++) omega.push_back(calc_omega_item<T>(len, i));
    for (size_t i = q; i < h; i++) {
      Cplx<T> t = omega[i - q];
      omega.push_back({t.im, -t.re});
    }
    for (size_t i = h; i < len; i++) {
      Cplx<T> t = omega[i - h];
      omega.push_back({-t.re, -t.im});
    }
  } else if ((len & 1) == 0) {
    size_t h = (len >> 1) > 1 ? (len >> 1) : 1;
    for (size_t i = 1; i < h; i++) omega.push_back(calc_omega_item<T>(len, i));
    for (size_t i = h; i < len; i++) {
      Cplx<T> t = omega[i - h];
      omega.push_back({-t.re, -t.im});
    }
  } else {
    for (size_t i = 1; i < len; i++) omega.push_back(calc_omega_item<T>(len, i));
  }
  omega.push_back(cone<T>());
  return omega;
}

// ---------------------------------------------------------------- a3/a4 digit reversal
// calc_bitreverse (src/precompute_utils.rs:70-91): mixed-radix digit-reversal
// gather list in factor order. `len` only sizes the allocation.
inline std::vector<size_t> calc_bitreverse(size_t len, const std::vector<Factor>& factors) {
  std::vector<size_t> ids;
  ids.reserve(len);
  size_t llen = 1;
  ids.push_back(0);
  for (const Factor& f : factors) {
    for (size_t c = 0; c < f.count; c++) {
      for (size_t j = 0; j < llen; j++) ids[j] *= f.value;
      for (size_t i = 1; i < f.value; i++)
        for (size_t j = 0; j < llen; j++) ids.push_back(ids[j] + i);
      llen *= f.value;
    }
  }
  return ids;
}

// calc_bitreverse2inplace (src/precompute_utils.rs:93-104), literal O(n^2)
// form: for each i, the position r >= i that currently holds source[i].
inline std::vector<size_t> calc_bitreverse2inplace_literal(const std::vector<size_t>& source) {
  std::vector<size_t> nums(source.size());
  for (size_t i = 0; i < nums.size(); i++) nums[i] = i;
  std::vector<size_t> out(source.size());
  for (size_t i = 0; i < source.size(); i++) {
    size_t r = i;
    while (nums[r] != source[i]) r++;
    std::swap(nums[i], nums[r]);
    out[i] = r;
  }
  return out;
}

// Same swap list in O(n): an inverse map replaces the linear search (the
// value source[i] sits at a unique position >= i because positions < i
// already hold source[0..i)). Tests check it equals the literal form.
inline std::vector<size_t> calc_bitreverse2inplace(const std::vector<size_t>& source) {
  size_t n = source.size();
  std::vector<size_t> nums(n), pos(n), out(n);
  for (size_t i = 0; i < n; i++) nums[i] = pos[i] = i;
  for (size_t i = 0; i < n; i++) {
    size_t r = pos[source[i]];
    size_t a = nums[i], b = nums[r];
    nums[i] = b;
    nums[r] = a;
    pos[b] = i;
    pos[a] = r;
    out[i] = r;
  }
  return out;
}

// ---------------------------------------------------------------- a7-a12 mixed radix
enum class Turn { Quarter, ThreeQuarter };
template <typename T> inline Cplx<T> turn(Turn t, Cplx<T> z) {
  return t == Turn::Quarter ? quarter_turn(z) : three_quarter_turn(z);
}

// mixed_kernel_radix2 (src/mixed_radix.rs:168-192)
template <typename T>
void radix2(Cplx<T>* ret, size_t count, size_t& po2, size_t& rad, const Cplx<T>* omega, size_t len) {
  for (size_t c = 0; c < count; c++) {
    size_t po2m = po2;
    po2 <<= 1;
    rad >>= 1;
    for (size_t j0 = 0; j0 < po2m; j0++) {
      Cplx<T> w1 = omega[rad * j0];
      for (size_t j = j0; j < len; j += po2) {
        size_t pos1 = j + po2m;
        Cplx<T> z1 = cmul(ret[pos1], w1);
        ret[pos1] = csub(ret[j], z1);
        ret[j] = cadd(ret[j], z1);
      }
    }
  }
}

// mixed_kernel_radix3 (src/mixed_radix.rs:194-228)
template <typename T>
void radix3(Cplx<T>* ret, size_t count, size_t& po2, size_t& rad, const Cplx<T>* omega, size_t len, Turn tf) {
  T t3scaler = tsin<T>(T(-2.0) * tpi<T>() / T(3.0));
  for (size_t c = 0; c < count; c++) {
    size_t po2m = po2;
    po2 *= 3;
    rad /= 3;
    for (size_t j0 = 0; j0 < po2m; j0++) {
      size_t wpos = rad * j0;
      Cplx<T> w1 = omega[wpos], w2 = omega[wpos << 1];
      for (size_t j = j0; j < len; j += po2) {
        size_t pos1 = j + po2m, pos2 = pos1 + po2m;
        Cplx<T> z1 = cmul(ret[pos1], w1);
        Cplx<T> z2 = cmul(ret[pos2], w2);
        Cplx<T> t1 = cadd(z1, z2);
        Cplx<T> t2 = csub(ret[j], cscale(t1, T(0.5)));
        Cplx<T> t3 = cscale(turn(tf, csub(z1, z2)), t3scaler);
        ret[j] = cadd(ret[j], t1);
        ret[pos1] = cadd(t2, t3);
        ret[pos2] = csub(t2, t3);
      }
    }
  }
}

// mixed_kernel_radix4 (src/mixed_radix.rs:230-270); also the pow2 engine of Chirp-Z.
template <typename T>
void radix4(Cplx<T>* ret, size_t count, size_t& po2, size_t& rad, const Cplx<T>* omega, size_t len, Turn tf) {
  for (size_t c = 0; c < count; c++) {
    size_t po2m = po2;
    po2 <<= 2;
    rad >>= 2;
    for (size_t j0 = 0; j0 < po2m; j0++) {
      size_t wpos = rad * j0;
      Cplx<T> w1 = omega[wpos], w2 = omega[wpos << 1], w3 = omega[wpos * 3];
      for (size_t j = j0; j < len; j += po2) {
        size_t pos1 = j + po2m, pos2 = pos1 + po2m, pos3 = pos2 + po2m;
        Cplx<T> wfa = ret[j];
        Cplx<T> wfc = cmul(ret[pos1], w1);
        Cplx<T> wfb = cmul(ret[pos2], w2);
        Cplx<T> wfd = cmul(ret[pos3], w3);
        Cplx<T> wfab = cadd(wfa, wfb), wfamb = csub(wfa, wfb);
        Cplx<T> wfcd = cadd(wfc, wfd);
        Cplx<T> wfcimdi = turn(tf, csub(wfc, wfd));
        ret[j] = cadd(wfab, wfcd);
        ret[pos1] = csub(wfamb, wfcimdi);
        ret[pos2] = csub(wfab, wfcd);
        ret[pos3] = cadd(wfamb, wfcimdi);
      }
    }
  }
}

// mixed_kernel_radix5 (src/mixed_radix.rs:272-334). The constants are
// recomputed inside the loop in the reference; they are loop invariant.
template <typename T>
void radix5(Cplx<T>* ret, size_t count, size_t& po2, size_t& rad, const Cplx<T>* omega, size_t len, Turn tf) {
  const T c_t6 = T(0.25) * tsqrt<T>(T(5.0));
  const T s04 = tsin<T>(T(-0.4) * tpi<T>());
  const T s02 = tsin<T>(T(-0.2) * tpi<T>());
  for (size_t c = 0; c < count; c++) {
    size_t po2m = po2;
    po2 *= 5;
    rad /= 5;
    for (size_t j0 = 0; j0 < po2m; j0++) {
      size_t wpos = rad * j0;
      Cplx<T> w1 = omega[wpos], w2 = omega[wpos << 1], w3 = omega[wpos * 3], w4 = omega[wpos << 2];
      for (size_t j = j0; j < len; j += po2) {
        size_t pos2 = j + po2m, pos3 = pos2 + po2m, pos4 = pos3 + po2m, pos5 = pos4 + po2m;
        Cplx<T> z0 = ret[j];
        Cplx<T> z1 = cmul(ret[pos2], w1), z2 = cmul(ret[pos3], w2);
        Cplx<T> z3 = cmul(ret[pos4], w3), z4 = cmul(ret[pos5], w4);
        Cplx<T> t1 = cadd(z1, z4), t2 = cadd(z2, z3), t3 = csub(z1, z4), t4 = csub(z2, z3);
        Cplx<T> t5 = cadd(t1, t2);
        Cplx<T> t6 = cscale(csub(t1, t2), c_t6);
        Cplx<T> t7 = csub(z0, cscale(t5, T(0.25)));
        Cplx<T> t8 = cadd(t6, t7), t9 = csub(t7, t6);
        Cplx<T> t10 = turn(tf, cadd(cscale(t3, s04), cscale(t4, s02)));
        Cplx<T> t11 = turn(tf, csub(cscale(t3, s02), cscale(t4, s04)));
        ret[j] = cadd(z0, t5);
        ret[pos2] = cadd(t8, t10);
        ret[pos3] = cadd(t9, t11);
        ret[pos4] = csub(t9, t11);
        ret[pos5] = csub(t8, t10);
      }
    }
  }
}

// mixed_kernel_other (src/mixed_radix.rs:336-368): definition DFT, O(r^2).
template <typename T>
void radix_other(Cplx<T>* ret, size_t value, size_t count, size_t& po2, size_t& rad, const Cplx<T>* omega,
                 size_t len) {
  size_t rot_width = len / value;
  std::vector<Cplx<T>> rot(value), z(value);
  std::vector<size_t> pos(value);
  for (size_t i = 0; i < value; i++) rot[i] = omega[rot_width * i];
  for (size_t c = 0; c < count; c++) {
    size_t po2m = po2;
    po2 *= value;
    rad /= value;
    for (size_t j0 = 0; j0 < po2m; j0++) {
      size_t wpos = rad * j0;
      for (size_t j = j0; j < len; j += po2) {
        for (size_t i = 0; i < value; i++) pos[i] = j + po2m * i;
        for (size_t i = 0; i < value; i++) z[i] = cmul(ret[pos[i]], omega[wpos * i]);
        for (size_t i = 0; i < value; i++) {
          Cplx<T> acc = z[0];
          for (size_t l = 1; l < value; l++) acc = cadd(acc, cmul(z[l], rot[(i * l) % value]));
          ret[pos[i]] = acc;
        }
      }
    }
  }
}

// fft_kernel (src/mixed_radix.rs:104-166): DIT stage loop over the factor list.
template <typename T>
void fft_kernel(Cplx<T>* src, size_t len, const Cplx<T>* omega, const std::vector<Factor>& factors, Turn tf) {
  size_t po2 = 1, rad = len;
  for (const Factor& f : factors) {
    switch (f.value) {
      case 2: radix2(src, f.count, po2, rad, omega, len); break;
      case 3: radix3(src, f.count, po2, rad, omega, len, tf); break;
      case 4: radix4(src, f.count, po2, rad, omega, len, tf); break;
      case 5: radix5(src, f.count, po2, rad, omega, len, tf); break;
      default: radix_other(src, f.value, f.count, po2, rad, omega, len); break;
    }
  }
}

template <typename T>
struct MixedRadixData {
  std::vector<size_t> ids;
  std::vector<Cplx<T>> omega, omega_back;
  std::vector<Factor> factors;
  std::vector<size_t> ids_inplace;
  bool has_inplace = false;
};

// convert_mixed (src/mixed_radix.rs:24-63): gather (with scale), then stages.
template <typename T>
std::vector<Cplx<T>> convert_mixed(const Cplx<T>* source, size_t len, bool is_back, T scaler,
                                   const MixedRadixData<T>& d) {
  std::vector<Cplx<T>> ret(len);
  if (scaler != T(1)) {
    for (size_t k = 0; k < len; k++) ret[k] = cscale(source[d.ids[k]], scaler);
  } else {
    for (size_t k = 0; k < len; k++) ret[k] = source[d.ids[k]];
  }
  if (is_back)
    fft_kernel(ret.data(), len, d.omega_back.data(), d.factors, Turn::ThreeQuarter);
  else
    fft_kernel(ret.data(), len, d.omega.data(), d.factors, Turn::Quarter);
  return ret;
}

// convert_mixed_inplace (src/mixed_radix.rs:65-102): swaps, stages, post-scale.
template <typename T>
void convert_mixed_inplace(Cplx<T>* source, size_t len, bool is_back, T scaler, const MixedRadixData<T>& d) {
  for (size_t i = 0; i < d.ids_inplace.size(); i++) {
    size_t s = d.ids_inplace[i];
    if (i != s) std::swap(source[i], source[s]);
  }
  if (is_back)
    fft_kernel(source, len, d.omega_back.data(), d.factors, Turn::ThreeQuarter);
  else
    fft_kernel(source, len, d.omega.data(), d.factors, Turn::Quarter);
  if (scaler != T(1))
    for (size_t i = 0; i < len; i++) source[i] = cscale(source[i], scaler);
}

// ---------------------------------------------------------------- a13/a14 Chirp-Z
template <typename T>
struct ChirpzData {
  size_t level = 0;
  std::vector<size_t> ids;
  std::vector<Cplx<T>> omega, omega_back, src_omega, rot_conj, rot_ft;
  T pow2len_inv = T(0);
};

// convert_rad2_inplace (src/chirpz.rs:27-85): swaps, optional 1/M pre-scale
// for the backward direction, one radix-2 pass when the level is odd, then
// level>>1 radix-4 passes.
template <typename T>
void convert_rad2_inplace(Cplx<T>* source, size_t slen, size_t level, const std::vector<size_t>& ids,
                          const Cplx<T>* omega, bool is_back, T pow2len_inv) {
  for (size_t i = 0; i < ids.size(); i++) {
    size_t s = ids[i];
    if (i != s) std::swap(source[i], source[s]);
  }
  if (is_back)
    for (size_t i = 0; i < slen; i++) source[i] = cscale(source[i], pow2len_inv);
  size_t po2 = 1, len = slen, rad = len;
  if ((level & 1) == 1) {
    rad >>= 1;
    po2 = 2;
    for (size_t j = 0; j < rad; j++) {
      size_t pa = j << 1, pb = pa + 1;
      Cplx<T> wfb = source[pb];
      source[pb] = csub(source[pa], wfb);
      source[pa] = cadd(source[pa], wfb);
    }
  }
  radix4(source, level >> 1, po2, rad, omega, len, is_back ? Turn::ThreeQuarter : Turn::Quarter);
}

// convert_chirpz / convert_chirpz_inplace (src/chirpz.rs:87-203): chirp
// multiply with index (i*i) % 2N, zero pad to M, FFT_M, x rot_ft, IFFT_M
// (1/M first), then x rot_conj[j]*scaler with j = i (forward) or N-i (back).
template <typename T>
void convert_chirpz(const Cplx<T>* source, Cplx<T>* out, size_t srclen, bool is_back, T scaler,
                    const ChirpzData<T>& d) {
  size_t len = size_t(1) << d.level, dlen = srclen << 1;
  std::vector<Cplx<T>> a(len, czero<T>());
  for (size_t i = 0; i < srclen; i++) a[i] = cmul(source[i], d.src_omega[(i * i) % dlen]);
  convert_rad2_inplace(a.data(), len, d.level, d.ids, d.omega.data(), false, d.pow2len_inv);
  for (size_t i = 0; i < len; i++) a[i] = cmul(a[i], d.rot_ft[i]);
  convert_rad2_inplace(a.data(), len, d.level, d.ids, d.omega_back.data(), true, d.pow2len_inv);
  for (size_t i = 0; i < srclen; i++) {
    size_t j = i == 0 ? 0 : (is_back ? srclen - i : i);
    out[i] = scaler != T(1) ? cmul(a[j], cscale(d.rot_conj[j], scaler)) : cmul(a[j], d.rot_conj[j]);
  }
}

// ---------------------------------------------------------------- a15 CFft1D
enum Method {
  FORWARD = 0, FORWARD0 = 1, FORWARDU = 2, FORWARDN = 3,
  BACKWARD = 4, BACKWARD0 = 5, BACKWARDU = 6, BACKWARDN = 7,
  FORWARD0I = 8, BACKWARD0I = 9, FORWARDUI = 10, BACKWARDUI = 11,
};

template <typename T>
class CFft1D {
 public:
  CFft1D() = default;
  explicit CFft1D(size_t len) { setup(len); }  // with_len (src/cfft1d.rs:83-92)

  // setup (src/cfft1d.rs:103-206): mixed radix when len is 7-smooth, else
  // Chirp-Z with M = next_pow2(len) << 1.
  void setup(size_t len) {
    const size_t MAX_PRIME = 7;
    len_ = len;
    scaler_n_ = T(1) / T(len);
    scaler_u_ = tsqrt<T>(scaler_n_);
    std::vector<Factor> factors = prime_factorization(len, MAX_PRIME);
    if (factors.empty()) {
      size_t pow2len = next_pow2(len) << 1;
      size_t lv = tz(pow2len);
      size_t dlen = len << 1;
      std::vector<Cplx<T>> src_omega = calc_omega<T>(dlen);
      std::vector<Cplx<T>> rot, rot_conj;
      rot.reserve(pow2len);
      rot_conj.reserve(pow2len);
      for (size_t i = 0; i < len; i++) {
        rot_conj.push_back(src_omega[(i * i) % dlen]);
        rot.push_back(src_omega[dlen - ((i * i) % dlen)]);
      }
      size_t hlen = (pow2len >> 1) + 1;
      for (size_t i = len; i < hlen; i++) {
        rot_conj.push_back(czero<T>());
        rot.push_back(czero<T>());
      }
      for (size_t i = hlen; i < pow2len; i++) {
        rot_conj.push_back(rot_conj[pow2len - i]);
        rot.push_back(rot[pow2len - i]);
      }
      // The level-match reuse branch (src/cfft1d.rs:142-160) keeps tables that
      // depend only on the level; rebuilding them gives identical values.
      ChirpzData<T> d;
      d.level = lv;
      d.ids = calc_bitreverse2inplace(calc_bitreverse(len, {{2, lv & 1}, {4, lv >> 1}}));
      d.omega = calc_omega<T>(pow2len);
      d.omega_back.assign(d.omega.rbegin(), d.omega.rend());
      d.pow2len_inv = T(1) / T(pow2len);
      convert_rad2_inplace(rot.data(), pow2len, lv, d.ids, d.omega.data(), false, d.pow2len_inv);
      d.src_omega = std::move(src_omega);
      d.rot_conj = std::move(rot_conj);
      d.rot_ft = std::move(rot);
      chirpz_ = std::move(d);
      mode_ = 2;
    } else {
      MixedRadixData<T> d;
      d.omega = calc_omega<T>(len);
      d.omega_back.assign(d.omega.rbegin(), d.omega.rend());
      d.ids = calc_bitreverse(len, factors);
      d.factors = factors;
      mixed_ = std::move(d);
      mode_ = 1;
    }
  }

  // convert (src/cfft1d.rs:208-230): len <= 1 copies; a new length re-plans.
  void convert(const Cplx<T>* src, Cplx<T>* dst, size_t len, bool is_back, T scaler) {
    if (len <= 1) {
      for (size_t i = 0; i < len; i++) dst[i] = src[i];
      return;
    }
    if (len != len_) setup(len);
    if (mode_ == 1) {
      std::vector<Cplx<T>> r = convert_mixed(src, len, is_back, scaler, mixed_);
      for (size_t i = 0; i < len; i++) dst[i] = r[i];
    } else {
      convert_chirpz(src, dst, len, is_back, scaler, chirpz_);
    }
  }

  // convert_inplace (src/cfft1d.rs:232-256): the swap list is built lazily.
  void convert_inplace(Cplx<T>* src, size_t len, bool is_back, T scaler) {
    if (len <= 1) return;
    if (len != len_) setup(len);
    if (mode_ == 1) {
      if (!mixed_.has_inplace) {
        mixed_.ids_inplace = calc_bitreverse2inplace(mixed_.ids);
        mixed_.has_inplace = true;
      }
      convert_mixed_inplace(src, len, is_back, scaler, mixed_);
    } else {
      std::vector<Cplx<T>> tmp(src, src + len);
      convert_chirpz(tmp.data(), src, len, is_back, scaler, chirpz_);
    }
  }

  // The 12 methods (src/cfft1d.rs:270-455) as (direction, scaler) pairs.
  void exec(Method m, const Cplx<T>* src, Cplx<T>* dst, size_t len) {
    if (len != len_ && len > 1) setup(len);
    switch (m) {
      case FORWARD: case FORWARD0: convert(src, dst, len, false, T(1)); break;
      case FORWARDU: convert(src, dst, len, false, scaler_u_); break;
      case FORWARDN: convert(src, dst, len, false, scaler_n_); break;
      case BACKWARD: case BACKWARDN: convert(src, dst, len, true, scaler_n_); break;
      case BACKWARD0: convert(src, dst, len, true, T(1)); break;
      case BACKWARDU: convert(src, dst, len, true, scaler_u_); break;
      case FORWARD0I: copy_then(src, dst, len), convert_inplace(dst, len, false, T(1)); break;
      case BACKWARD0I: copy_then(src, dst, len), convert_inplace(dst, len, true, T(1)); break;
      case FORWARDUI: copy_then(src, dst, len), convert_inplace(dst, len, false, scaler_u_); break;
      case BACKWARDUI: copy_then(src, dst, len), convert_inplace(dst, len, true, scaler_u_); break;
    }
  }

  void forward0i(Cplx<T>* x, size_t len) { convert_inplace(x, len, false, T(1)); }
  void backward0i(Cplx<T>* x, size_t len) { convert_inplace(x, len, true, T(1)); }
  void forward0(const Cplx<T>* s, Cplx<T>* d, size_t len) { convert(s, d, len, false, T(1)); }
  void backward0(const Cplx<T>* s, Cplx<T>* d, size_t len) { convert(s, d, len, true, T(1)); }

  size_t len() const { return len_; }
  int mode() const { return mode_; }
  const MixedRadixData<T>& mixed() const { return mixed_; }
  const ChirpzData<T>& chirpz() const { return chirpz_; }

 private:
  static void copy_then(const Cplx<T>* src, Cplx<T>* dst, size_t len) {
    if (src != dst)
      for (size_t i = 0; i < len; i++) dst[i] = src[i];
  }
  size_t len_ = 0;
  T scaler_n_ = T(0), scaler_u_ = T(0);
  int mode_ = 0;  // 0 none, 1 mixed radix, 2 chirp-z
  MixedRadixData<T> mixed_;
  ChirpzData<T> chirpz_;
};

// ---------------------------------------------------------------- a16 CFft2D
// CFft2D::convert (src/cfft2d.rs:327-363): row FFTs of length N scattered
// into work[N][M], then column FFTs of length M gathered into ret[M][N] and
// multiplied by the scaler. `src`/`dst` are row-major M x N.
// fft_m is built for len_m but applied to rows of length len_n, so it
// re-plans on first use when M != N (src/cfft2d.rs:99, src/cfft1d.rs:216-218).
template <typename T>
class CFft2D {
 public:
  CFft2D(size_t m, size_t n) : m_(m), n_(n), fft_m_(m ? m : 1), fft_n_(n ? n : 1), work_(n * m), row_(n), col_(m) {}

  void convert(const Cplx<T>* src, Cplx<T>* dst, size_t m, size_t n, bool is_back, T scaler) {
    if (m == 0 || n == 0) return;
    for (size_t i = 0; i < m; i++) {
      if (is_back)
        fft_m_.backward0(src + i * n, row_.data(), n);
      else
        fft_m_.forward0(src + i * n, row_.data(), n);
      for (size_t j = 0; j < n; j++) work_[j * m + i] = row_[j];
    }
    for (size_t i = 0; i < n; i++) {
      if (is_back)
        fft_n_.backward0(&work_[i * m], col_.data(), m);
      else
        fft_n_.forward0(&work_[i * m], col_.data(), m);
      for (size_t j = 0; j < m; j++) dst[j * n + i] = cscale(col_[j], scaler);
    }
  }

 private:
  size_t m_, n_;
  CFft1D<T> fft_m_, fft_n_;
  std::vector<Cplx<T>> work_, row_, col_;
};

// ---------------------------------------------------------------- a17 RFft1D
template <typename T>
class RFft1D {
 public:
  // new (src/rfft1d.rs:73-90) and calc_rfft_coef (src/rfft1d.rs:44-65).
  explicit RFft1D(size_t len) {
    if (len & 1) throw std::invalid_argument("invalid length");
    len_ = len;
    fft_.setup(len >> 1);
    scaler_n_ = T(1) / T(len);
    scaler_u_ = tsqrt<T>(scaler_n_);
    std::vector<Cplx<T>> omega = calc_omega<T>(len);
    for (size_t i = 0; i < (len >> 1); i++)
      coef_.push_back(cscale(cadd(Cplx<T>{T(1), T(0)}, cmul_i(omega[i])), T(0.5)));
    for (size_t i = 0; i < (len >> 1); i++)
      bcoef_.push_back(cscale(csub(Cplx<T>{T(1), T(0)}, cmul_i(omega[len - i])), T(0.5)));
    work_.assign(len >> 1, czero<T>());
  }

  // convert (src/rfft1d.rs:115-151): pack, in-place half FFT, split.
  void forward(const T* src, Cplx<T>* ret, T scaler) {
    size_t t = len_ >> 1;
    for (size_t i = 0; i < t; i++) work_[i] = cscale(Cplx<T>{src[i << 1], src[(i << 1) + 1]}, scaler);
    fft_.forward0i(work_.data(), t);
    size_t hlen = (len_ + 1) >> 1, qlen = (len_ + 3) >> 2;
    for (size_t i = 0; i <= t; i++) ret[i] = czero<T>();
    for (size_t i = 1; i < qlen; i++) {
      Cplx<T> x = cmul(coef_[i], csub(work_[i], cconj(work_[hlen - i])));
      ret[i] = csub(work_[i], x);
      ret[hlen - i] = cadd(work_[hlen - i], cconj(x));
    }
    ret[0] = {work_[0].re + work_[0].im, T(0)};
    if (tz(len_) >= 2) ret[qlen] = cconj(work_[qlen]);
    ret[hlen] = {work_[0].re - work_[0].im, T(0)};
  }

  // convert_back (src/rfft1d.rs:153-187): merge, in-place half IFFT, unpack x2.
  void backward(const Cplx<T>* src, T* ret, T scaler) {
    scaler = scaler * T(2.0);
    size_t hlen = (len_ + 1) >> 1, qlen = (len_ + 3) >> 2;
    work_[0] = cscale(Cplx<T>{src[0].re + src[hlen].re, src[0].re - src[hlen].re}, T(0.5));
    if (tz(len_) >= 2) work_[qlen] = cconj(src[qlen]);
    for (size_t i = 1; i < qlen; i++) {
      Cplx<T> x = cmul(bcoef_[i], csub(src[i], cconj(src[hlen - i])));
      work_[i] = csub(src[i], x);
      work_[hlen - i] = cadd(src[hlen - i], cconj(x));
    }
    fft_.backward0i(work_.data(), len_ >> 1);
    for (size_t i = 0; i < hlen; i++) {
      ret[2 * i] = work_[i].re * scaler;
      ret[2 * i + 1] = work_[i].im * scaler;
    }
  }

  T scaler_n() const { return scaler_n_; }
  T scaler_u() const { return scaler_u_; }

 private:
  CFft1D<T> fft_;
  size_t len_ = 0;
  std::vector<Cplx<T>> coef_, bcoef_, work_;
  T scaler_n_ = T(0), scaler_u_ = T(0);
};

// ---------------------------------------------------------------- a18 Dct1D
template <typename T>
class Dct1D {
 public:
  // Dct1D::new / Dct2Worker1D::setup / Dct3Worker1D::setup
  // (src/dct1d.rs:53-62, :200-226, :323-349).
  Dct1D(int type, size_t len, bool is_ortho) {
    if (len & 1) throw std::invalid_argument("invalid length");
    type_ = type;
    len_ = len;
    cfft_.setup(len >> 1);
    std::vector<Cplx<T>> o4 = calc_omega<T>(len << 2);
    std::vector<Cplx<T>> o1 = calc_omega<T>(len);
    if (type == 2) {
      for (size_t i = 0; i < (len >> 1) + 1; i++) omega_.push_back(o4[(len << 2) - i]);
      for (size_t i = 0; i < (len >> 1); i++)
        coef_.push_back(cscale(cadd(Cplx<T>{T(1), T(0)}, cmul_i(o1[i])), T(0.5)));
      ortho_scaler_ = is_ortho ? tsqrt<T>(T(0.5)) : T(1);
    } else {
      for (size_t i = 0; i < (len >> 1) + 1; i++) omega_.push_back(o4[i]);
      for (size_t i = 0; i < (len >> 1); i++)
        coef_.push_back(cscale(csub(Cplx<T>{T(1), T(0)}, cmul_i(o1[len - i])), T(0.5)));
      ortho_scaler_ = is_ortho ? tsqrt<T>(T(0.5)) : T(0.5);
    }
    work_.assign(len >> 1, czero<T>());
    unitary_scaler_ = tsqrt<T>(T(2.0) / T(len));
  }

  void convert(const T* src, T* ret, T scaler) {
    if (type_ == 2)
      dct2(src, ret, scaler);
    else
      dct3(src, ret, scaler);
  }
  T unitary_scaler() const { return unitary_scaler_; }

 private:
  // Dct2Worker1D::convert (src/dct1d.rs:236-290)
  void dct2(const T* source, T* ret, T scaler) {
    size_t hlen = len_ >> 1, qlen = hlen >> 1;
    if (qlen == 0) {
      work_[0] = cscale(Cplx<T>{source[0] * ortho_scaler_, source[1]}, scaler);
    } else {
      work_[0] = cscale(Cplx<T>{source[0] * ortho_scaler_, source[2]}, scaler);
      for (size_t i = 1; i < qlen; i++) work_[i] = cscale(Cplx<T>{source[i << 2], source[(i << 2) + 2]}, scaler);
      for (size_t i = 0; i < qlen; i++)
        work_[hlen - i - 1] = cscale(Cplx<T>{source[(i << 2) + 3], source[(i << 2) + 1]}, scaler);
      if (hlen & 1) work_[qlen] = cscale(Cplx<T>{source[len_ - 2], source[len_ - 1]}, scaler);
    }
    cfft_.forward0i(work_.data(), hlen);
    for (size_t i = 0; i < len_; i++) ret[i] = T(0);
    size_t q2 = (len_ + 3) >> 2;
    for (size_t i = 1; i < q2; i++) {
      Cplx<T> wconj = cconj(work_[hlen - i]);
      Cplx<T> x = cmul(coef_[i], csub(work_[i], wconj));
      Cplx<T> j = cmul(cconj(csub(work_[i], x)), omega_[i]);
      ret[i] = j.re;
      ret[len_ - i] = j.im;
      Cplx<T> k = cmul(cadd(wconj, x), omega_[hlen - i]);
      ret[hlen - i] = k.re;
      ret[hlen + i] = k.im;
    }
    if (tz(len_) >= 2) {
      Cplx<T> x = cmul(work_[q2], omega_[q2]);
      ret[q2] = x.re;
      ret[len_ - q2] = x.im;
    }
    ret[0] = work_[0].re + work_[0].im;
    ret[hlen] = (work_[0].re - work_[0].im) * omega_[hlen].re;
  }

  // Dct3Worker1D::convert (src/dct1d.rs:359-409)
  void dct3(const T* source, T* ret, T scaler) {
    size_t hlen = len_ >> 1;
    T zval = source[0] * ortho_scaler_;
    T hval = source[hlen] * omega_[hlen].re;
    work_[0] = cscale(Cplx<T>{zval + hval, zval - hval}, scaler);
    size_t qlen = (len_ + 3) >> 2;
    if (tz(len_) >= 2)
      work_[qlen] = cmul(Cplx<T>{source[qlen], source[len_ - qlen]}, cscale(omega_[qlen], scaler));
    for (size_t i = 1; i < qlen; i++) {
      Cplx<T> j = cconj(cscale(cmul(Cplx<T>{source[i], source[len_ - i]}, omega_[i]), scaler));
      Cplx<T> k = cscale(cmul(Cplx<T>{source[hlen - i], source[hlen + i]}, omega_[hlen - i]), scaler);
      Cplx<T> x = cmul(coef_[i], csub(j, k));
      work_[i] = csub(j, x);
      work_[hlen - i] = cadd(cconj(k), cconj(x));
    }
    cfft_.backward0i(work_.data(), hlen);
    size_t q = hlen >> 1, o = 0;
    for (size_t i = 0; i < q; i++) {
      ret[o++] = work_[i].re;
      ret[o++] = work_[hlen - i - 1].im;
      ret[o++] = work_[i].im;
      ret[o++] = work_[hlen - i - 1].re;
    }
    if (hlen & 1) {
      ret[o++] = work_[q].re;
      ret[o++] = work_[q].im;
    }
  }

  int type_ = 2;
  size_t len_ = 0;
  CFft1D<T> cfft_;
  std::vector<Cplx<T>> omega_, coef_, work_;
  T ortho_scaler_ = T(1), unitary_scaler_ = T(1);
};

// ---------------------------------------------------------------- a19 Mdct1D
// sine_window / vorbis_window (src/mdct1d.rs:42-53)
template <typename T> inline T sine_window(size_t l, size_t p) {
  return tsin<T>(tpi<T>() * (T(p) + T(0.5)) / T(l));
}
template <typename T> inline T vorbis_window(size_t l, size_t p) {
  T s = tsin<T>(tpi<T>() * (T(p) + T(0.5)) / T(l));
  return tsin<T>(s * s * tpi<T>() * T(0.5));
}

template <typename T>
class Mdct1D {
 public:
  // Mdct1D::new with a window table evaluated at setup (src/mdct1d.rs:62-95, :102-111).
  Mdct1D(const T* window, size_t len) {
    if (len & 3) throw std::invalid_argument("invalid length");
    len_ = len;
    fft_.setup(len >> 2);
    scaler_u_ = T(1) / tsqrt<T>(T(len >> 1));
    scaler_ui_ = tsqrt<T>(T(len >> 1));
    T sc = tsqrt<T>(tsqrt<T>(T(2.0) / T(len)));
    for (size_t i = 0; i < (len >> 2); i++) twiddle_.push_back(cscale(calc_omega_item<T>(len << 3, (i << 3) + 1), sc));
    win_.assign(window, window + len);
    work_.assign(len >> 2, czero<T>());
  }

  T scaler_u() const { return scaler_u_; }
  T scaler_ui() const { return scaler_ui_; }

  // Mdct1D::convert (src/mdct1d.rs:197-241)
  void forward(const T* source, T* ret, T scaler) {
    size_t lenh = len_ >> 1, lenq = lenh >> 1, leno = lenq - (lenq >> 1);
    size_t len3q = lenh + lenq, len5q = lenh + len3q;
    const T* w = win_.data();
    for (size_t i = 0; i < leno; i++) {
      size_t n = i << 1;
      work_[i] = cmul(Cplx<T>{source[len3q - 1 - n] * w[len3q - 1 - n] + source[len3q + n] * w[len3q + n],
                              source[lenq + n] * w[lenq + n] - source[lenq - 1 - n] * w[lenq - 1 - n]},
                      twiddle_[i]);
    }
    for (size_t i = leno; i < lenq; i++) {
      size_t n = i << 1;
      work_[i] = cmul(Cplx<T>{source[len3q - 1 - n] * w[len3q - 1 - n] - source[n - lenq] * w[n - lenq],
                              source[lenq + n] * w[lenq + n] + source[len5q - 1 - n] * w[len5q - 1 - n]},
                      twiddle_[i]);
    }
    fft_.forward0i(work_.data(), lenq);
    for (size_t i = 0; i < lenq; i++) {
      size_t n = i << 1;
      Cplx<T> t = cmul(work_[i], cscale(twiddle_[i], scaler));
      ret[n] = -t.re;
      ret[lenh - 1 - n] = t.im;
    }
  }

  // Mdct1D::convert_back (src/mdct1d.rs:243-291): pre-twiddle x(-2), FORWARD FFT.
  void backward(const T* source, T* ret, T scaler) {
    size_t lenh = len_ >> 1, lenq = lenh >> 1, leno = lenq - (lenq >> 1);
    size_t len3q = lenh + lenq, len5q = lenh + len3q;
    const T* w = win_.data();
    for (size_t i = 0; i < lenq; i++) {
      size_t n = i << 1;
      work_[i] = cmul(Cplx<T>{source[n], source[lenh - 1 - n]}, cscale(twiddle_[i], T(-2.0)));
    }
    fft_.forward0i(work_.data(), lenq);
    for (size_t i = 0; i < len_; i++) ret[i] = T(0);
    for (size_t i = 0; i < leno; i++) {
      size_t n = i << 1;
      Cplx<T> t = cmul(work_[i], cscale(twiddle_[i], scaler));
      ret[len3q - 1 - n] = t.re * w[len3q - 1 - n];
      ret[len3q + n] = t.re * w[len3q + n];
      ret[lenq + n] = -t.im * w[lenq + n];
      ret[lenq - 1 - n] = t.im * w[lenq - 1 - n];
    }
    for (size_t i = leno; i < lenq; i++) {
      size_t n = i << 1;
      Cplx<T> t = cmul(work_[i], cscale(twiddle_[i], scaler));
      ret[len3q - 1 - n] = t.re * w[len3q - 1 - n];
      ret[n - lenq] = -t.re * w[n - lenq];
      ret[lenq + n] = -t.im * w[lenq + n];
      ret[len5q - 1 - n] = -t.im * w[len5q - 1 - n];
    }
  }

 private:
  size_t len_ = 0;
  CFft1D<T> fft_;
  std::vector<Cplx<T>> twiddle_, work_;
  std::vector<T> win_;
  T scaler_u_ = T(0), scaler_ui_ = T(0);
};

}  // namespace chfft_oracle
