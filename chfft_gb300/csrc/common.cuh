// Shared device helpers: interleaved complex arithmetic, compile-time roots
// of unity and the register-resident DFT butterflies used by every kernel.
//
// Complex data is interleaved {re, im} (float2 / double2), the layout of
// num-complex's #[repr(C)] Complex<T> that the reference API passes around
// (src/cfft1d.rs:270 takes &[Complex<T>]).
#pragma once

// The kernel headers also compile under NVRTC (plan-time specialised
// kernels), which provides the CUDA vector types itself.
#ifndef __CUDACC_RTC__
#include <cuda_runtime.h>
#include <stdint.h>
#endif

#define CHFFT_HD __host__ __device__ __forceinline__

namespace chfft {

template <class A, class B> struct same_type { static constexpr bool value = false; };
template <class A> struct same_type<A, A> { static constexpr bool value = true; };

template <typename T> struct Cx;
template <> struct Cx<float> { using type = float2; };
template <> struct Cx<double> { using type = double2; };
template <typename T> using cx_t = typename Cx<T>::type;

template <typename C> struct Real;
template <> struct Real<float2> { using type = float; };
template <> struct Real<double2> { using type = double; };

CHFFT_HD float2 mk(float a, float b) { return make_float2(a, b); }
CHFFT_HD double2 mk(double a, double b) { return make_double2(a, b); }

template <typename C> CHFFT_HD C cadd(C a, C b) { return mk(a.x + b.x, a.y + b.y); }
template <typename C> CHFFT_HD C csub(C a, C b) { return mk(a.x - b.x, a.y - b.y); }
template <typename C> CHFFT_HD C cmul(C a, C b) { return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
// a * conj(b)
template <typename C> CHFFT_HD C cmulc(C a, C b) { return mk(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); }
template <typename C, typename R> CHFFT_HD C cscale(C a, R s) { return mk(a.x * s, a.y * s); }
template <typename C> CHFFT_HD C cconj(C a) { return mk(a.x, -a.y); }
template <typename C> CHFFT_HD C czero() {
  using R = typename Real<C>::type;
  return mk(R(0), R(0));
}
// a * (-i) and a * i
template <typename C> CHFFT_HD C mul_mi(C a) { return mk(a.y, -a.x); }
template <typename C> CHFFT_HD C mul_pi(C a) { return mk(-a.y, a.x); }

// ---------------------------------------------------------------------------
// Compile-time cos/sin of 2*pi*k/R, from the Taylor series after reducing the
// angle to [0, pi/4] with the octant symmetries. Used only for the constant
// roots of unity inside the butterflies; tables are generated at run time.
namespace ct {
constexpr double kPi = 3.141592653589793238462643383279502884;
__host__ __device__ constexpr double taylor_sin(double x) {
  double term = x, sum = x, x2 = x * x;
  for (int n = 1; n < 16; n++) {
    term = -term * x2 / double((2 * n) * (2 * n + 1));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr double taylor_cos(double x) {
  double term = 1.0, sum = 1.0, x2 = x * x;
  for (int n = 1; n < 16; n++) {
    term = -term * x2 / double((2 * n - 1) * (2 * n));
    sum += term;
  }
  return sum;
}
// cos and sin of 2*pi*k/r, exact octant reduction on the integer numerator.
__host__ __device__ constexpr double cos2pi(long k, long r) {
  k %= r;
  if (k < 0) k += r;
  // angle = 2*pi*k/r = (pi/4) * (8k/r); octant o = floor(8k/r)
  long num = 8 * k;
  long o = num / r;
  long rem = num - o * r;  // angle within the octant = (pi/4) * rem / r
  double a = (kPi / 4.0) * double(rem) / double(r);
  double b = (kPi / 4.0) * double(r - rem) / double(r);  // pi/4 - a
  switch (o) {
    case 0: return taylor_cos(a);
    case 1: return taylor_sin(b);
    case 2: return -taylor_sin(a);
    case 3: return -taylor_cos(b);
    case 4: return -taylor_cos(a);
    case 5: return -taylor_sin(b);
    case 6: return taylor_sin(a);
    default: return taylor_cos(b);
  }
}
__host__ __device__ constexpr double sin2pi(long k, long r) { return cos2pi(k * 4 - r, 4 * r); }  // sin t = cos(t - pi/2)
}  // namespace ct

// w = exp(-2*pi*i*e/R) multiplied into v at compile time, with the exact
// quarter-turn cases (1, -i, -1, i) done without a multiply.
template <int R, int E, typename C>
CHFFT_HD C twiddle_const(C v) {
  using Rl = typename Real<C>::type;
  constexpr int e = ((E % R) + R) % R;
  if constexpr (e == 0) {
    return v;
  } else if constexpr (4 * e == R) {
    return mul_mi(v);
  } else if constexpr (2 * e == R) {
    return mk(-v.x, -v.y);
  } else if constexpr (4 * e == 3 * R) {
    return mul_pi(v);
  } else if constexpr (8 * e == R) {  // (1 - i)/sqrt2
    constexpr Rl h = Rl(0.70710678118654752440084436210484903);
    return mk((v.x + v.y) * h, (v.y - v.x) * h);
  } else if constexpr (8 * e == 3 * R) {  // (-1 - i)/sqrt2
    constexpr Rl h = Rl(0.70710678118654752440084436210484903);
    return mk((v.y - v.x) * h, -(v.x + v.y) * h);
  } else {
    constexpr Rl c = Rl(ct::cos2pi(e, R));
    constexpr Rl s = Rl(-ct::sin2pi(e, R));
    return mk(v.x * c - v.y * s, v.x * s + v.y * c);
  }
}

// ---------------------------------------------------------------------------
// Forward DFT of R points held in registers, y_k = sum_n x_n w^{nk},
// w = exp(-2*pi*i/R). In place on v[0..R).
template <int R> struct Dft;

template <> struct Dft<1> {
  template <typename C> CHFFT_HD static void run(C*) {}
};

template <> struct Dft<2> {
  template <typename C> CHFFT_HD static void run(C* v) {
    C a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <> struct Dft<3> {
  template <typename C> CHFFT_HD static void run(C* v) {
    using Rl = typename Real<C>::type;
    constexpr Rl s = Rl(0.86602540378443864676372317075293618);  // sin(2pi/3)
    C t1 = cadd(v[1], v[2]);
    C t2 = mk(v[0].x - Rl(0.5) * t1.x, v[0].y - Rl(0.5) * t1.y);
    C d = csub(v[1], v[2]);
    C t3 = mk(s * d.y, -s * d.x);  // -i * s * (x1 - x2)
    v[0] = cadd(v[0], t1);
    v[1] = cadd(t2, t3);
    v[2] = csub(t2, t3);
  }
};

template <> struct Dft<4> {
  template <typename C> CHFFT_HD static void run(C* v) {
    C t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
    C t2 = cadd(v[1], v[3]), t3 = mul_mi(csub(v[1], v[3]));
    v[0] = cadd(t0, t2);
    v[2] = csub(t0, t2);
    v[1] = cadd(t1, t3);
    v[3] = csub(t1, t3);
  }
};

template <> struct Dft<5> {
  template <typename C> CHFFT_HD static void run(C* v) {
    using Rl = typename Real<C>::type;
    constexpr Rl c1 = Rl(ct::cos2pi(1, 5)), c2 = Rl(ct::cos2pi(2, 5));
    constexpr Rl s1 = Rl(ct::sin2pi(1, 5)), s2 = Rl(ct::sin2pi(2, 5));
    C t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
    C t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
    C x0 = v[0];
    v[0] = cadd(x0, cadd(t1, t2));
    C a1 = mk(x0.x + c1 * t1.x + c2 * t2.x, x0.y + c1 * t1.y + c2 * t2.y);
    C a2 = mk(x0.x + c2 * t1.x + c1 * t2.x, x0.y + c2 * t1.y + c1 * t2.y);
    C b1 = mk(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y);
    C b2 = mk(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y);
    // y1 = a1 - i b1, y4 = a1 + i b1, y2 = a2 - i b2, y3 = a2 + i b2
    v[1] = mk(a1.x + b1.y, a1.y - b1.x);
    v[4] = mk(a1.x - b1.y, a1.y + b1.x);
    v[2] = mk(a2.x + b2.y, a2.y - b2.x);
    v[3] = mk(a2.x - b2.y, a2.y + b2.x);
  }
};

template <> struct Dft<7> {
  template <typename C> CHFFT_HD static void run(C* v) {
    using Rl = typename Real<C>::type;
    constexpr Rl c1 = Rl(ct::cos2pi(1, 7)), c2 = Rl(ct::cos2pi(2, 7)), c3 = Rl(ct::cos2pi(3, 7));
    constexpr Rl s1 = Rl(ct::sin2pi(1, 7)), s2 = Rl(ct::sin2pi(2, 7)), s3 = Rl(ct::sin2pi(3, 7));
    C t1 = cadd(v[1], v[6]), u1 = csub(v[1], v[6]);
    C t2 = cadd(v[2], v[5]), u2 = csub(v[2], v[5]);
    C t3 = cadd(v[3], v[4]), u3 = csub(v[3], v[4]);
    C x0 = v[0];
    v[0] = cadd(x0, cadd(t1, cadd(t2, t3)));
    // m = 1: cos (c1,c2,c3), sin (s1,s2,s3); m = 2: (c2,c3,c1), (s2,-s3,-s1);
    // m = 3: (c3,c1,c2), (s3,-s1,s2)
    C a1 = mk(x0.x + c1 * t1.x + c2 * t2.x + c3 * t3.x, x0.y + c1 * t1.y + c2 * t2.y + c3 * t3.y);
    C a2 = mk(x0.x + c2 * t1.x + c3 * t2.x + c1 * t3.x, x0.y + c2 * t1.y + c3 * t2.y + c1 * t3.y);
    C a3 = mk(x0.x + c3 * t1.x + c1 * t2.x + c2 * t3.x, x0.y + c3 * t1.y + c1 * t2.y + c2 * t3.y);
    C b1 = mk(s1 * u1.x + s2 * u2.x + s3 * u3.x, s1 * u1.y + s2 * u2.y + s3 * u3.y);
    C b2 = mk(s2 * u1.x - s3 * u2.x - s1 * u3.x, s2 * u1.y - s3 * u2.y - s1 * u3.y);
    C b3 = mk(s3 * u1.x - s1 * u2.x + s2 * u3.x, s3 * u1.y - s1 * u2.y + s2 * u3.y);
    v[1] = mk(a1.x + b1.y, a1.y - b1.x);
    v[6] = mk(a1.x - b1.y, a1.y + b1.x);
    v[2] = mk(a2.x + b2.y, a2.y - b2.x);
    v[5] = mk(a2.x - b2.y, a2.y + b2.x);
    v[3] = mk(a3.x + b3.y, a3.y - b3.x);
    v[4] = mk(a3.x - b3.y, a3.y + b3.x);
  }
};

// Composite R = A*B (A the divisor nearest sqrt(R)): with n = q + A*p and
// k = k1 + B*k2, y_k = sum_q w_A^{q k2} w_R^{q k1} sum_p x_{q+Ap} w_B^{p k1}.
template <int R> __host__ __device__ constexpr int split_a() {
  int best = 1;
  for (int a = 2; a * a <= R; a++)
    if (R % a == 0) best = a;
  return best;
}

template <int R> struct Dft {
  static constexpr int A = split_a<R>();
  static constexpr int B = R / A;
  static_assert(A > 1, "prime radix without a dedicated butterfly");

  template <int Q, typename C> CHFFT_HD static void inner(C* v) {
    if constexpr (Q < A) {
      C t[B];
#pragma unroll
      for (int p = 0; p < B; p++) t[p] = v[Q + A * p];
      Dft<B>::run(t);
      twid<Q, 0>(t);
#pragma unroll
      for (int k1 = 0; k1 < B; k1++) v[Q + A * k1] = t[k1];
      inner<Q + 1>(v);
    }
  }
  template <int Q, int K1, typename C> CHFFT_HD static void twid(C* t) {
    if constexpr (K1 < B) {
      t[K1] = twiddle_const<R, Q * K1>(t[K1]);
      twid<Q, K1 + 1>(t);
    }
  }
  template <typename C> CHFFT_HD static void run(C* v) {
    inner<0>(v);
    C y[R];
#pragma unroll
    for (int k1 = 0; k1 < B; k1++) {
      C t[A];
#pragma unroll
      for (int q = 0; q < A; q++) t[q] = v[q + A * k1];
      Dft<A>::run(t);
#pragma unroll
      for (int k2 = 0; k2 < A; k2++) y[k1 + B * k2] = t[k2];
    }
#pragma unroll
    for (int k = 0; k < R; k++) v[k] = y[k];
  }
};

}  // namespace chfft
