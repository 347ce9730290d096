// Double-float real: a value hi + lo held as two FP32 numbers with
// |lo| <= ulp(hi)/2 (about 48 significant bits), computed on the FP32 pipe.
// GB300 executes FP64 at a small fraction of its FP32 rate, so a propagator
// march that needs FP64-level accuracy runs faster in this arithmetic than in
// native FP64 (SCFT_PREC_DF).
//
// Algorithms (Dekker 1971; Knuth, TAOCP vol. 2, 4.2.2; the "sloppy" pair
// addition of Hida, Li & Bailey, QD library paper, 2001):
//   TwoSum(a, b)     = (s, e), s = fl(a + b), a + b = s + e exactly
//   FastTwoSum(a, b) = (s, e), the same when |a| >= |b|
//   TwoProd(a, b)    = (p, e), p = fl(a * b), e = fma(a, b, -p) exactly
//   (ah, al) + (bh, bl): (s, e) = TwoSum(ah, bh); e += al + bl; FastTwoSum(s, e)
//   (ah, al) * (bh, bl): (p, e) = TwoProd(ah, bh); e += ah*bl + al*bh; FastTwoSum(p, e)
// The addition's error is bounded relative to |a| + |b| (not to |a + b|),
// which is the normwise accuracy an FFT needs.  None of these sequences may
// be reassociated; plain IEEE compilation (no fast-math) keeps them, and the
// products use explicit fmaf.
#pragma once

#include <math.h>

namespace scft {

struct __align__(8) dfloat {
  float hi, lo;
  __host__ __device__ constexpr dfloat() : hi(0.f), lo(0.f) {}
  __host__ __device__ constexpr dfloat(float h, float l) : hi(h), lo(l) {}
  // rounds d to the nearest pair: hi = fl32(d), lo = fl32(d - hi)
  __host__ __device__ constexpr dfloat(double d)
      : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

struct __align__(16) dfloat2 {
  dfloat x, y;
};

__host__ __device__ __forceinline__ dfloat df_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return dfloat(s, (a - (s - bb)) + (b - bb));
}
__host__ __device__ __forceinline__ dfloat df_fast_two_sum(float a, float b) {
  const float s = a + b;
  return dfloat(s, b - (s - a));
}

__host__ __device__ __forceinline__ dfloat operator-(dfloat a) { return dfloat(-a.hi, -a.lo); }
__host__ __device__ __forceinline__ dfloat operator+(dfloat a, dfloat b) {
  const dfloat s = df_two_sum(a.hi, b.hi);
  return df_fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
__host__ __device__ __forceinline__ dfloat operator-(dfloat a, dfloat b) { return a + (-b); }
__host__ __device__ __forceinline__ dfloat operator*(dfloat a, dfloat b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df_fast_two_sum(p, e);
}
// a + b and a - b without the final renormalisation (8 instead of 11
// instructions): the pair may carry |lo| above ulp(hi)/2, the value is still
// hi + lo and the error stays bounded relative to |a| + |b| (a few ulps of
// 2^-48 more per chained addition).  For the short chains of butterfly
// additions inside a DFT codelet: every product renormalises.
__host__ __device__ __forceinline__ dfloat df_add_lazy(dfloat a, dfloat b) {
  const dfloat s = df_two_sum(a.hi, b.hi);
  return dfloat(s.hi, s.lo + (a.lo + b.lo));
}
__host__ __device__ __forceinline__ dfloat df_sub_lazy(dfloat a, dfloat b) {
  const dfloat s = df_two_sum(a.hi, -b.hi);
  return dfloat(s.hi, s.lo + (a.lo - b.lo));
}
// a*b + c*d with one renormalisation (19 instead of 25 instructions as two
// products and a sum): the high products exactly (TwoProd), their sum exactly
// (TwoSum), every low term added in FP32.
__host__ __device__ __forceinline__ dfloat df_dot2(dfloat a, dfloat b, dfloat c, dfloat d) {
  const float p = a.hi * b.hi, q = c.hi * d.hi;
  const float ep = fmaf(a.hi, b.hi, -p), eq = fmaf(c.hi, d.hi, -q);
  const dfloat s = df_two_sum(p, q);
  float lo = s.lo + (ep + eq);
  lo = fmaf(a.hi, b.lo, lo);
  lo = fmaf(a.lo, b.hi, lo);
  lo = fmaf(c.hi, d.lo, lo);
  lo = fmaf(c.lo, d.hi, lo);
  return df_fast_two_sum(s.hi, lo);
}
__host__ __device__ __forceinline__ dfloat &operator+=(dfloat &a, dfloat b) { return a = a + b; }
__host__ __device__ __forceinline__ dfloat &operator-=(dfloat &a, dfloat b) { return a = a - b; }
__host__ __device__ __forceinline__ dfloat &operator*=(dfloat &a, dfloat b) { return a = a * b; }

#if defined(__CUDACC__)
// Loads through the read-only path for the element types of the kernels.
template <typename X> __device__ __forceinline__ X ldg(const X *p) { return __ldg(p); }
template <> __device__ __forceinline__ dfloat ldg<dfloat>(const dfloat *p) {
  const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
  return dfloat(v.x, v.y);
}
template <> __device__ __forceinline__ dfloat2 ldg<dfloat2>(const dfloat2 *p) {
  const float4 v = __ldg(reinterpret_cast<const float4 *>(p));
  dfloat2 r;
  r.x = dfloat(v.x, v.y);
  r.y = dfloat(v.z, v.w);
  return r;
}
#endif

}  // namespace scft
