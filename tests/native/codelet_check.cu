// Host-side check of the in-register DFT codelets (scft_ver1.01_gb300/csrc/fft_reg.cuh)
// against a naive long-double DFT.  Built and run on the CPU by tests/test_codelets_cpu.py.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "fft_reg.cuh"

using namespace scft;

template <typename C> double rel_err_one(int R, bool inv, const C *in, const C *out) {
  double num = 0, den = 0;
  for (int k = 0; k < R; ++k) {
    long double re = 0, im = 0;
    for (int n = 0; n < R; ++n) {
      long double ang = (inv ? 2.0L : -2.0L) * 3.141592653589793238462643383279L * n * k / R;
      re += (long double)in[n].x * cosl(ang) - (long double)in[n].y * sinl(ang);
      im += (long double)in[n].x * sinl(ang) + (long double)in[n].y * cosl(ang);
    }
    double dx = (double)(out[k].x - re), dy = (double)(out[k].y - im);
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
    printf("R=%3d %s %s max_rel_err=%.3e\n", R, sizeof(T) == 4 ? "f32" : "f64",
           inv ? "inv" : "fwd", worst);
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

int main() {
  srand(12345);
  int bad = check_all<double2>(1e-14) + check_all<float2>(2e-6);
  printf(bad ? "FAIL %d\n" : "OK\n", bad);
  return bad ? 1 : 0;
}
