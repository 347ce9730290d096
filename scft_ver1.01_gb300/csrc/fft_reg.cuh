// In-register DFT codelets for compile-time sizes (FP32 / FP64 complex).
//
// dft<R, INV>(v): v[k] <- sum_n v[n] * exp(-+2 pi i n k / R) in place, natural
// order in and out, INV selecting the + sign (unnormalised inverse).  Sizes
// 2, 3, 4, 5 are written out; composite sizes use one Cooley-Tukey split
// R = A*B (input n = n1 + A*n2, output k = B*k1 + k2) with twiddles that are
// compile-time constants.  The twiddle values come from constexpr Taylor
// series evaluated by the compiler in double precision.
#pragma once

#include <type_traits>

#include "common.cuh"

namespace scft {
namespace reg {

constexpr double kPi = 3.14159265358979323846264338327950288;

// Taylor series on [-pi, pi] (the argument is reduced exactly from m/n).
constexpr double cx_sin(double x) {
  double x2 = x * x, term = x, sum = x;
  for (int i = 1; i < 24; ++i) {
    term *= -x2 / ((2.0 * i) * (2.0 * i + 1.0));
    sum += term;
  }
  return sum;
}
constexpr double cx_cos(double x) {
  double x2 = x * x, term = 1.0, sum = 1.0;
  for (int i = 1; i < 24; ++i) {
    term *= -x2 / ((2.0 * i - 1.0) * (2.0 * i));
    sum += term;
  }
  return sum;
}
// angle 2*pi*m/n reduced to [-pi, pi]
constexpr double cx_angle(long m, long n) {
  m %= n;
  if (m < 0) m += n;
  if (2 * m > n) m -= n;
  return 2.0 * kPi * (double)m / (double)n;
}
constexpr double cos2pi(long m, long n) { return cx_cos(cx_angle(m, n)); }
constexpr double sin2pi(long m, long n) { return cx_sin(cx_angle(m, n)); }

template <int I, int N, typename F>
__host__ __device__ __forceinline__ void static_for(F &&f) {
  if constexpr (I < N) {
    f(std::integral_constant<int, I>{});
    static_for<I + 1, N>(f);
  }
}

template <typename C> struct real_of;
template <> struct real_of<float2> { typedef float type; };
template <> struct real_of<double2> { typedef double type; };
template <> struct real_of<dfloat2> { typedef dfloat type; };

// Butterfly additions: for the double-float pair without renormalisation
// (df_add_lazy: the codelet's products renormalise).
template <typename C> __host__ __device__ __forceinline__ C badd(C a, C b) { return cadd(a, b); }
template <typename C> __host__ __device__ __forceinline__ C bsub(C a, C b) { return csub(a, b); }
template <> __host__ __device__ __forceinline__ dfloat2 badd(dfloat2 a, dfloat2 b) {
  dfloat2 r;
  r.x = df_add_lazy(a.x, b.x);
  r.y = df_add_lazy(a.y, b.y);
  return r;
}
template <> __host__ __device__ __forceinline__ dfloat2 bsub(dfloat2 a, dfloat2 b) {
  dfloat2 r;
  r.x = df_sub_lazy(a.x, b.x);
  r.y = df_sub_lazy(a.y, b.y);
  return r;
}
// v * (c + i s)
template <typename C, typename T> __host__ __device__ __forceinline__ C rot(C v, T c, T s) {
  return mkc<C, T>(v.x * c - v.y * s, v.x * s + v.y * c);
}
__host__ __device__ __forceinline__ dfloat2 rot(dfloat2 v, dfloat c, dfloat s) {
  dfloat2 r;
  r.x = df_dot2(v.x, c, v.y, -s);
  r.y = df_dot2(v.x, s, v.y, c);
  return r;
}

// v * exp(-/+ 2 pi i m / R), exact for multiples of a quarter turn.
template <int M, int R, bool INV, typename C>
__host__ __device__ __forceinline__ C twmul(C v) {
  typedef typename real_of<C>::type T;
  constexpr int m = ((M % R) + R) % R;
  if constexpr (m == 0) {
    return v;
  } else if constexpr (4 * m == R) {          // -i (forward) / +i (inverse)
    return INV ? mkc<C, T>(-v.y, v.x) : mkc<C, T>(v.y, -v.x);
  } else if constexpr (2 * m == R) {
    return mkc<C, T>(-v.x, -v.y);
  } else if constexpr (4 * m == 3 * R) {      // +i (forward) / -i (inverse)
    return INV ? mkc<C, T>(v.y, -v.x) : mkc<C, T>(-v.y, v.x);
  } else {
    constexpr T c = (T)cos2pi(m, R);
    constexpr T s = INV ? (T)sin2pi(m, R) : (T)-sin2pi(m, R);
    return rot(v, c, s);
  }
}

template <int R> constexpr int split_factor() {
  return (R % 4 == 0 && R != 4) ? 4 : (R % 2 == 0 ? 2 : (R % 3 == 0 ? 3 : 5));
}

template <int R, bool INV, typename C>
__host__ __device__ __forceinline__ void dft(C *v) {
  typedef typename real_of<C>::type T;
  if constexpr (R == 1) {
  } else if constexpr (R == 2) {
    C a = v[0], b = v[1];
    v[0] = badd(a, b);
    v[1] = bsub(a, b);
  } else if constexpr (R == 3) {
    constexpr T s3 = (T)0.866025403784438646763723170752936183;
    C a = v[0], b = v[1], c = v[2];
    C s = badd(b, c), d = bsub(b, c);
    v[0] = badd(a, s);
    C m = mkc<C, T>(a.x - T(0.5) * s.x, a.y - T(0.5) * s.y);
    // forward: -i*s3*d ; inverse: +i*s3*d
    C t = INV ? mkc<C, T>(-s3 * d.y, s3 * d.x) : mkc<C, T>(s3 * d.y, -s3 * d.x);
    v[1] = badd(m, t);
    v[2] = bsub(m, t);
  } else if constexpr (R == 4) {
    C a = badd(v[0], v[2]), b = bsub(v[0], v[2]);
    C c = badd(v[1], v[3]), e = bsub(v[1], v[3]);
    C d = INV ? mkc<C, T>(-e.y, e.x) : mkc<C, T>(e.y, -e.x);
    v[0] = badd(a, c);
    v[2] = bsub(a, c);
    v[1] = badd(b, d);
    v[3] = bsub(b, d);
  } else if constexpr (R == 5) {
    constexpr T c1 = (T)0.309016994374947424102293417182819059;   // cos(2pi/5)
    constexpr T c2 = (T)-0.809016994374947424102293417182819059;  // cos(4pi/5)
    constexpr T s1 = (T)0.951056516295153572116439333379382143;   // sin(2pi/5)
    constexpr T s2 = (T)0.587785252292473129168705954639072769;   // sin(4pi/5)
    C a = v[0];
    C p1 = badd(v[1], v[4]), d1 = bsub(v[1], v[4]);
    C p2 = badd(v[2], v[3]), d2 = bsub(v[2], v[3]);
    v[0] = badd(a, badd(p1, p2));
    C m1 = mkc<C, T>(a.x + c1 * p1.x + c2 * p2.x, a.y + c1 * p1.y + c2 * p2.y);
    C m2 = mkc<C, T>(a.x + c2 * p1.x + c1 * p2.x, a.y + c2 * p1.y + c1 * p2.y);
    T t1x = s1 * d1.x + s2 * d2.x, t1y = s1 * d1.y + s2 * d2.y;
    T t2x = s2 * d1.x - s1 * d2.x, t2y = s2 * d1.y - s1 * d2.y;
    if (INV) { t1x = -t1x; t1y = -t1y; t2x = -t2x; t2y = -t2y; }
    v[1] = mkc<C, T>(m1.x + t1y, m1.y - t1x);
    v[4] = mkc<C, T>(m1.x - t1y, m1.y + t1x);
    v[2] = mkc<C, T>(m2.x + t2y, m2.y - t2x);
    v[3] = mkc<C, T>(m2.x - t2y, m2.y + t2x);
  } else {
    constexpr int A = split_factor<R>();
    constexpr int B = R / A;
    static_assert(A * B == R, "unsupported codelet size");
    C t[A][B];
    static_for<0, A>([&](auto n1_) {
      constexpr int n1 = decltype(n1_)::value;
      static_for<0, B>([&](auto n2_) {
        constexpr int n2 = decltype(n2_)::value;
        t[n1][n2] = v[n1 + A * n2];
      });
      dft<B, INV>(t[n1]);
      static_for<1, B>([&](auto k2_) {
        constexpr int k2 = decltype(k2_)::value;
        t[n1][k2] = twmul<n1 * k2, R, INV>(t[n1][k2]);
      });
    });
    static_for<0, B>([&](auto k2_) {
      constexpr int k2 = decltype(k2_)::value;
      C u[A];
      static_for<0, A>([&](auto n1_) {
        constexpr int n1 = decltype(n1_)::value;
        u[n1] = t[n1][k2];
      });
      dft<A, INV>(u);
      static_for<0, A>([&](auto k1_) {
        constexpr int k1 = decltype(k1_)::value;
        v[B * k1 + k2] = u[k1];
      });
    });
  }
}

}  // namespace reg
}  // namespace scft
