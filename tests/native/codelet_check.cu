// Host-side check of the in-register DFT codelets (scft_ver1.01_gb300/csrc/fft_reg.cuh)
// against a naive long-double DFT.  Built and run on the CPU by tests/test_codelets_cpu.py.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "fft_reg.cuh"

using namespace scft;

static long double ld(float x) { return x; }
static long double ld(double x) { return x; }
static long double ld(dfloat x) { return (long double)x.hi + (long double)x.lo; }
template <typename T> const char *label() { return sizeof(T) == 4 ? "f32" : "f64"; }
template <> const char *label<dfloat>() { return "df "; }

template <typename C> double rel_err_one(int R, bool inv, const C *in, const C *out) {
  double num = 0, den = 0;
  for (int k = 0; k < R; ++k) {
    long double re = 0, im = 0;
    for (int n = 0; n < R; ++n) {
      long double ang = (inv ? 2.0L : -2.0L) * 3.141592653589793238462643383279L * n * k / R;
      re += ld(in[n].x) * cosl(ang) - ld(in[n].y) * sinl(ang);
      im += ld(in[n].x) * sinl(ang) + ld(in[n].y) * cosl(ang);
    }
    double dx = (double)(ld(out[k].x) - re), dy = (double)(ld(out[k].y) - im);
    num = fmax(num, sqrt(dx * dx + dy * dy));
    den = fmax(den, (double)sqrtl(re * re + im * im));
  }
  return num / den;
}

template <int R, typename C> int check(double tol) {
  typedef typename reg::real_of<C>::type T;
  int bad = 0;
  for (int inv = 0; inv < 2; ++inv) {
    double worst = 0;
    for (int trial = 0; trial < 20; ++trial) {
      C in[R], v[R];
      for (int i = 0; i < R; ++i) {
        in[i].x = (T)(rand() / (double)RAND_MAX - 0.5);
        in[i].y = (T)(rand() / (double)RAND_MAX - 0.5);
        v[i] = in[i];
      }
      if (inv) reg::dft<R, true>(v);
      else reg::dft<R, false>(v);
      worst = fmax(worst, rel_err_one(R, inv, in, v));
    }
    printf("R=%3d %s %s max_rel_err=%.3e\n", R, label<T>(), inv ? "inv" : "fwd", worst);
    if (!(worst < tol)) bad++;
  }
  return bad;
}

template <typename C> int check_all(double tol) {
  int bad = 0;
  bad += check<2, C>(tol); bad += check<3, C>(tol); bad += check<4, C>(tol);
  bad += check<5, C>(tol); bad += check<6, C>(tol); bad += check<8, C>(tol);
  bad += check<10, C>(tol); bad += check<12, C>(tol); bad += check<16, C>(tol);
  bad += check<20, C>(tol); bad += check<24, C>(tol); bad += check<32, C>(tol);
  return bad;
}

// Double-float arithmetic against long double: the sum within 2^-44 of
// |a| + |b|, the product within 2^-44 of |a b|, the unrenormalised sums and
// the two-product dot within 2^-44 normwise (random pairs over a wide
// exponent range, either sign).
int check_dfloat_ops() {
  int bad = 0;
  double worst_add = 0, worst_mul = 0;
  for (int t = 0; t < 200000; ++t) {
    const double x = (rand() / (double)RAND_MAX - 0.5) * ldexp(1.0, rand() % 40 - 20);
    const double y = (rand() / (double)RAND_MAX - 0.5) * ldexp(1.0, rand() % 40 - 20);
    const dfloat a(x), b(y);
    const long double A = ld(a), B = ld(b);
    const long double s = ld(a + b), p = ld(a * b), d = ld(a - b);
    worst_add = fmax(worst_add, (double)(fabsl(s - (A + B)) / (fabsl(A) + fabsl(B))));
    worst_add = fmax(worst_add, (double)(fabsl(d - (A - B)) / (fabsl(A) + fabsl(B))));
    if (A * B != 0) worst_mul = fmax(worst_mul, (double)(fabsl(p - A * B) / fabsl(A * B)));
    // the unrenormalised butterfly additions and the two-product dot
    // (normwise: relative to |a| + |b|, |ab| + |cd|)
    const long double l = ld(df_add_lazy(a, b)), ls = ld(df_sub_lazy(a, b));
    worst_add = fmax(worst_add, (double)(fabsl(l - (A + B)) / (fabsl(A) + fabsl(B))));
    worst_add = fmax(worst_add, (double)(fabsl(ls - (A - B)) / (fabsl(A) + fabsl(B))));
    {
      const dfloat c(y * 0.37 + x), d(x * 1.3 - y);
      const long double C = ld(c), D = ld(d), ref = A * B + C * D;
      const long double nrm = fabsl(A * B) + fabsl(C * D);
      if (nrm != 0)
        worst_mul = fmax(worst_mul, (double)(fabsl(ld(df_dot2(a, b, c, d)) - ref) / nrm));
    }
    // the pair is normalised: |lo| <= ulp(hi)/2
    const dfloat r = a * b;
    if (fabsf(r.lo) > 0.5f * fabsf(nextafterf(r.hi, INFINITY) - r.hi) * 1.0000001f) bad++;
  }
  printf("dfloat add/sub max rel err %.3e, mul %.3e, unnormalised %d\n", worst_add, worst_mul,
         bad);
  const double lim = ldexp(1.0, -44);
  return bad + (worst_add < lim ? 0 : 1) + (worst_mul < lim ? 0 : 1);
}

int main() {
  srand(12345);
  int bad = check_all<double2>(1e-14) + check_all<float2>(2e-6) + check_dfloat_ops() +
            check_all<dfloat2>(1e-12);
  printf(bad ? "FAIL %d\n" : "OK\n", bad);
  return bad ? 1 : 0;
}
