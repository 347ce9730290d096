// Cubic interpolating spline of the reference's spline.c / spline.h: the
// Forsythe, Malcolm & Moler (1977) SPLINE / SEVAL construction (symmetric
// tridiagonal system for sigma_i = S''(x_i)/6, end conditions from the third
// derivatives of the cubics through the first and last four knots) with the
// optional known end slopes of the reference (end1/end2 = 1).  The host
// functions keep the reference's order of floating-point operations, so their
// coefficients and values are bit-identical to it on the same machine (this
// file is compiled with FP contraction off); the device evaluator uses
// explicitly rounded operations and matches the host evaluation bit for bit.
//
// Layout of the result, as in the reference (spline.c:28-95): for knots
// x[0..n-1] (strictly increasing) and y[0..n-1],
//   S(u) = y[i] + b[i] w + c[i] w^2 + d[i] w^3,  w = u - x[i],  x[i] <= u <= x[i+1],
// with b, c, d of length n (the last entries continue the last segment).
#include <cuda_runtime.h>

#include "scft_capi.h"

namespace {

// Segment of u: the hint `last` is kept while x[last] <= u <= x[last+1],
// else a bisection picks i with x[i] <= u < x[i+1] (0 below the first knot,
// n-1 at or above the last) -- the reference's search (spline.c:254-270).
__host__ __device__ inline int find_segment(int n, double u, const double *x, int last) {
  int i = last;
  if (i >= n - 1 || i < 0) i = 0;
  if (x[i] > u || x[i + 1] < u) {
    int lo = 0, hi = n;
    do {
      const int mid = (lo + hi) / 2;
      if (u < x[mid]) hi = mid;
      if (u >= x[mid]) lo = mid;
    } while (hi > lo + 1);
    i = lo;
  }
  return i;
}

// Explicitly rounded arithmetic: no contraction into FMA on either side.
__host__ __device__ inline double add(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
__host__ __device__ inline double mul(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}

__host__ __device__ inline double value_at(int i, double u, const double *x, const double *y,
                                           const double *b, const double *c, const double *d) {
  const double w = add(u, -x[i]);
  return add(y[i], mul(w, add(b[i], mul(w, add(c[i], mul(w, d[i]))))));
}
__host__ __device__ inline double slope_at(int i, double u, const double *x, const double *b,
                                           const double *c, const double *d) {
  const double w = add(u, -x[i]);
  return add(b[i], mul(w, add(mul(2.0, c[i]), mul(mul(w, 3.0), d[i]))));
}
// integral over [x[i], x[i] + w] of segment i
__host__ __device__ inline double piece_integral(int i, double w, const double *y,
                                                 const double *b, const double *c,
                                                 const double *d) {
  const double third = c[i] / 3.0;
  return mul(w, add(y[i], mul(w, add(mul(0.5, b[i]),
                                     mul(w, add(third, mul(mul(w, 0.25), d[i])))))));
}
__host__ __device__ inline double integral_to(int i, double u, const double *x, const double *y,
                                              const double *b, const double *c,
                                              const double *d) {
  double sum = 0.0;
  for (int j = 0; j < i; ++j) sum = add(sum, piece_integral(j, add(x[j + 1], -x[j]), y, b, c, d));
  return add(sum, piece_integral(i, add(u, -x[i]), y, b, c, d));
}

__global__ void k_spline_eval(int n, const double *__restrict__ x, const double *__restrict__ y,
                              const double *__restrict__ b, const double *__restrict__ c,
                              const double *__restrict__ d, const double *__restrict__ u,
                              double *__restrict__ out, long long count, int mode) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count;
       k += (long long)gridDim.x * blockDim.x) {
    const double uk = u[k];
    const int i = find_segment(n, uk, x, 0);
    out[k] = mode == 0 ? value_at(i, uk, x, y, b, c, d)
           : mode == 1 ? slope_at(i, uk, x, b, c, d)
                       : integral_to(i, uk, x, y, b, c, d);
  }
}

}  // namespace

extern "C" {

int scft_spline(int n, int end1, int end2, double slope1, double slope2, const double *x,
                const double *y, double *b, double *c, double *d, int *iflag) {
  if (!iflag) return SCFT_ERR_INVALID_ARG;
  *iflag = 0;
  if (n < 2) {            // cannot interpolate
    *iflag = 1;
    return SCFT_OK;
  }
  if (!x || !y || !b || !c || !d) return SCFT_ERR_INVALID_ARG;
  for (int i = 1; i < n; ++i)
    if (x[i] <= x[i - 1]) {
      *iflag = 2;         // abscissas not strictly increasing
      return SCFT_OK;
    }
  const int last = n - 1;
  if (n == 2) {           // one linear segment
    b[0] = (y[1] - y[0]) / (x[1] - x[0]);
    c[0] = d[0] = 0.0;
    b[1] = b[0];
    c[1] = d[1] = 0.0;
    return SCFT_OK;
  }
  // Symmetric tridiagonal system: b = diagonal, d = off-diagonal (interval
  // lengths), c = right-hand side (differences of divided differences).
  d[0] = x[1] - x[0];
  c[1] = (y[1] - y[0]) / d[0];
  for (int i = 1; i < last; ++i) {
    d[i] = x[i + 1] - x[i];
    b[i] = 2.0 * (d[i - 1] + d[i]);
    c[i + 1] = (y[i + 1] - y[i]) / d[i];
    c[i] = c[i + 1] - c[i];
  }
  // End rows: the third derivative of the cubic through the first (last)
  // four knots; with three knots, a constant third derivative (zero rhs).
  b[0] = -d[0];
  b[last] = -d[n - 2];
  c[0] = 0.0;
  c[last] = 0.0;
  if (n > 3) {
    const double e0 = c[2] / (x[3] - x[1]) - c[1] / (x[2] - x[0]);
    const double en = c[n - 2] / (x[last] - x[n - 3]) - c[n - 3] / (x[n - 2] - x[n - 4]);
    c[0] = e0 * d[0] * d[0] / (x[3] - x[0]);
    c[last] = -en * d[n - 2] * d[n - 2] / (x[last] - x[n - 4]);
  }
  // Known end slopes replace the end rows.
  if (end1 == 1) {
    b[0] = 2.0 * (x[1] - x[0]);
    c[0] = (y[1] - y[0]) / (x[1] - x[0]) - slope1;
  }
  if (end2 == 1) {
    b[last] = 2.0 * (x[last] - x[n - 2]);
    c[last] = slope2 - (y[last] - y[n - 2]) / (x[last] - x[n - 2]);
  }
  // Gaussian elimination without pivoting, then back substitution: c = sigma.
  for (int i = 1; i < n; ++i) {
    const double t = d[i - 1] / b[i - 1];
    b[i] = b[i] - t * d[i - 1];
    c[i] = c[i] - t * c[i - 1];
  }
  c[last] = c[last] / b[last];
  for (int i = n - 2; i >= 0; --i) c[i] = (c[i] - d[i] * c[i + 1]) / b[i];
  // Polynomial coefficients of each segment.
  b[last] = (y[last] - y[n - 2]) / d[n - 2] + d[n - 2] * (c[n - 2] + 2.0 * c[last]);
  for (int i = 0; i < last; ++i) {
    b[i] = (y[i + 1] - y[i]) / d[i] - d[i] * (c[i + 1] + 2.0 * c[i]);
    d[i] = (c[i + 1] - c[i]) / d[i];
    c[i] = 3.0 * c[i];
  }
  c[last] = 3.0 * c[last];
  d[last] = d[n - 2];
  return SCFT_OK;
}

double scft_spline_eval(int n, double u, const double *x, const double *y, const double *b,
                        const double *c, const double *d, int *last) {
  const int i = find_segment(n, u, x, last ? *last : 0);
  if (last) *last = i;
  return value_at(i, u, x, y, b, c, d);
}

double scft_spline_deriv(int n, double u, const double *x, const double *b, const double *c,
                         const double *d, int *last) {
  const int i = find_segment(n, u, x, last ? *last : 0);
  if (last) *last = i;
  return slope_at(i, u, x, b, c, d);
}

double scft_spline_integral(int n, double u, const double *x, const double *y, const double *b,
                            const double *c, const double *d, int *last) {
  const int i = find_segment(n, u, x, last ? *last : 0);
  if (last) *last = i;
  return integral_to(i, u, x, y, b, c, d);
}

int scft_spline_eval_device(int n, const double *x, const double *y, const double *b,
                            const double *c, const double *d, const double *u, double *out,
                            long long count, int mode, void *stream) {
  if (n < 2 || !x || !y || !b || !c || !d || !u || !out || count < 0 || mode < 0 || mode > 2)
    return SCFT_ERR_INVALID_ARG;
  if (count == 0) return SCFT_OK;
  long long blocks = (count + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  k_spline_eval<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      n, x, y, b, c, d, u, out, count, mode);
  return cudaGetLastError() == cudaSuccess ? SCFT_OK : SCFT_ERR_CUDA;
}

}  // extern "C"
