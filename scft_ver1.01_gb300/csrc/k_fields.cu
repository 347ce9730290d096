// Field kernels of the SCF iteration: Boltzmann factors, propagator
// hand-offs, deterministic per-instance reductions (mean subtraction, Q, free
// energy), the trapezoid contour sum giving phi, and simple mixing.
// All reductions are two-level and in a fixed order, so results are
// bit-reproducible from run to run.
#include <string.h>

#include "common.cuh"
#include "kernels.h"

namespace scft {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ double block_sum(double v, double *sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (wid == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;  // valid in thread 0
}
__device__ __forceinline__ double block_max(double v, double *sh) {
  v = warp_max(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (wid == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    r = warp_max(r);
  }
  __syncthreads();
  return r;
}

// initilize_wdz (cuda_aid.cu:254): W = exp(-w*ds2).  The FP32 factor is
// evaluated in FP32 (GB300's FP64 pipe is narrow; the result is rounded to
// FP32 anyway).
template <typename R>
__global__ void k_boltzmann(const double *__restrict__ w, R *__restrict__ W, long long n,
                            double ds2) {
  stream_loop<4>(n, [&](long long i) { return w[i]; }, [&](long long i, double x) {
    if constexpr (sizeof(R) == 4) W[i] = expf(-(float)x * (float)ds2);
    else W[i] = exp(-x * ds2);
  });
}

template <typename R>
__global__ void k_fill(R *__restrict__ x, long long n, R v, long long bs) {
  R *xb = x + blockIdx.y * bs;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    xb[i] = v;
}

template <typename R, typename D>
__global__ void k_copy(D *__restrict__ dst, long long dbs, const R *__restrict__ src,
                       long long sbs, long long M) {
  D *d = dst + blockIdx.y * dbs;
  const R *s = src + blockIdx.y * sbs;
  stream_loop<4>(M, [&](long long i) { return s[i]; }, [&](long long i, R x) { d[i] = (D)x; });
}

template <typename R>
__global__ void k_partial_sum(const R *__restrict__ x, long long bs, long long M,
                              double *__restrict__ partial) {
  __shared__ double sh[32];
  const R *xb = x + blockIdx.y * bs;
  double acc = 0.0;
  stream_loop<8>(M, [&](long long i) { return xb[i]; },
                 [&](long long, R x) { acc += (double)x; });
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) partial[blockIdx.y * gridDim.x + blockIdx.x] = acc;
}

__global__ void k_finalize_sum(const double *__restrict__ partial, int nblk, double scale,
                               double *__restrict__ out) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) acc += partial[blockIdx.x * nblk + i];
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) out[blockIdx.x] = acc * scale;
}

__global__ void k_minus_average(double *__restrict__ data, const double *__restrict__ sum,
                                long long M) {
  double *d = data + blockIdx.y * M;
  // minus_average (cuda_aid.cu:377) divides per element; the quotient is the
  // same for every element, so it is formed once per block (bit-identical
  // result; an FP64 division per thread costs more than the whole pass).
  __shared__ double s_mean;
  if (threadIdx.x == 0) s_mean = sum[blockIdx.y] / (double)M;
  __syncthreads();
  const double mean = s_mean;
  stream_loop<8>(M, [&](long long i) { return d[i]; },
                 [&](long long i, double x) { d[i] = x - mean; });
}

__global__ void k_q_ffl(const double *__restrict__ sum, long long M, double ds0, int batch,
                        double *__restrict__ Q, double *__restrict__ ffl) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < batch) {
    const double q = sum[b] / (double)M;  // cuda_scft.cu:124
    Q[b] = q;
    ffl[b] = ds0 / q;                      // cuda_scft.cu:125
  }
}

// Trapezoid contour sum (w_to_phi_go, cuda_aid.cu:87-112).  q, qc are
// contour-outer [b][s][M].  FP64 accumulation for double; for float the
// products are accumulated with a compensated (TwoSum) FP32 pair, which keeps
// ~FP64-level summation error without GB300's slow FP64 pipe.
// cw: the block's contour weights (contour_weights below); the reference's
// trapezoid is m = ns, c_odd = c_even = 1 and the ends listed with 1/2.
template <typename R>
__global__ void k_contour_phi(const R *__restrict__ q, const R *__restrict__ qc, int ns,
                              long long M, const double *__restrict__ ffl,
                              double *__restrict__ phi, ContourWeights cw);

template <>
__global__ void k_contour_phi<double>(const double *__restrict__ q, const double *__restrict__ qc,
                                      int ns, long long M, const double *__restrict__ ffl,
                                      double *__restrict__ phi, ContourWeights cw) {
  const int b = blockIdx.y;
  const long long qbs = (long long)(ns + 1) * M;
  const double *qb = q + b * qbs, *qcb = qc + b * qbs;
  const bool trap = cw.c_odd == 1.0 && cw.c_even == 1.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < M;
       i += (long long)gridDim.x * blockDim.x) {
    // special points before the interior (s = 0), in the reference's order
    double acc = 0.0;
    int k = 0;
    for (; k < cw.nspec && cw.s[k] < 1; ++k) acc += cw.w[k] * qb[cw.s[k] * M + i] * qcb[cw.s[k] * M + i];
    if (trap) {
      for (int s = 1; s < cw.m; ++s) acc += qb[s * M + i] * qcb[s * M + i];
    } else {
      double ao = 0.0, ae = 0.0;
      for (int s = 1; s < cw.m; ++s) {
        const double pr = qb[s * M + i] * qcb[s * M + i];
        if (s & 1) ao += pr;
        else ae += pr;
      }
      acc += cw.c_odd * ao + cw.c_even * ae;
    }
    for (; k < cw.nspec; ++k) acc += cw.w[k] * qb[cw.s[k] * M + i] * qcb[cw.s[k] * M + i];
    phi[b * M + i] = acc * ffl[b];
  }
}

template <>
__global__ void k_contour_phi<float>(const float *__restrict__ q, const float *__restrict__ qc,
                                     int ns, long long M, const double *__restrict__ ffl,
                                     double *__restrict__ phi, ContourWeights cw) {
  const int b = blockIdx.y;
  const long long qbs = (long long)(ns + 1) * M;
  const float *qb = q + b * qbs, *qcb = qc + b * qbs;
  const bool trap = cw.c_odd == 1.0 && cw.c_even == 1.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < M;
       i += (long long)gridDim.x * blockDim.x) {
    // interior: compensated FP32 sums, one per weight class
    float hi = 0.f, lo = 0.f, hi2 = 0.f, lo2 = 0.f;
    if (trap) {
      for (int s = 1; s < cw.m; ++s) {
        // the product rounded on its own (no FMA contraction into the sum):
        // TwoSum needs the addend it adds
        const float p = __fmul_rn(qb[s * M + i], qcb[s * M + i]);
        float e;
        two_sum(hi, p, hi, e);
        lo += e;
      }
    } else {
      for (int s = 1; s < cw.m; ++s) {
        const float p = __fmul_rn(qb[s * M + i], qcb[s * M + i]);
        float e;
        if (s & 1) {
          two_sum(hi, p, hi, e);
          lo += e;
        } else {
          two_sum(hi2, p, hi2, e);
          lo2 += e;
        }
      }
    }
    // the listed points in FP64
    double ends = 0.0;
    for (int k = 0; k < cw.nspec; ++k)
      ends += cw.w[k] * ((double)qb[cw.s[k] * M + i] * (double)qcb[cw.s[k] * M + i]);
    const double inner = trap ? (double)hi + (double)lo
                              : cw.c_odd * ((double)hi + (double)lo) +
                                    cw.c_even * ((double)hi2 + (double)lo2);
    phi[b * M + i] = (inner + ends) * ffl[b];
  }
}

// Double-float propagators: products and sums in pair arithmetic (FP32 pipe),
// one conversion to FP64 per point.
template <>
__global__ void k_contour_phi<dfloat>(const dfloat *__restrict__ q, const dfloat *__restrict__ qc,
                                      int ns, long long M, const double *__restrict__ ffl,
                                      double *__restrict__ phi, ContourWeights cw) {
  const int b = blockIdx.y;
  const long long qbs = (long long)(ns + 1) * M;
  const dfloat *qb = q + b * qbs, *qcb = qc + b * qbs;
  const bool trap = cw.c_odd == 1.0 && cw.c_even == 1.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < M;
       i += (long long)gridDim.x * blockDim.x) {
    dfloat ao, ae;
    for (int s = 1; s < cw.m; ++s) {
      const dfloat pr = qb[s * M + i] * qcb[s * M + i];
      if (trap || (s & 1)) ao += pr;
      else ae += pr;
    }
    double ends = 0.0;
    for (int k = 0; k < cw.nspec; ++k)
      ends += cw.w[k] * ((double)qb[cw.s[k] * M + i] * (double)qcb[cw.s[k] * M + i]);
    const double inner = trap ? (double)ao : cw.c_odd * (double)ao + cw.c_even * (double)ae;
    phi[b * M + i] = (inner + ends) * ffl[b];
  }
}

__global__ void k_phi_w(double *__restrict__ wa, double *__restrict__ wb,
                        const double *__restrict__ pha, const double *__restrict__ phb,
                        double hAB, double wopt, double wcmp, long long n) {
  stream_loop<4>(n, [&](long long i) { return dquad{wa[i], wb[i], pha[i], phb[i]}; },
                 [&](long long i, dquad v) {
    // phi_w, cuda_aid.cu:398-412
    const double a = v.x, b = v.y, pa = v.z, pb = v.w;
    const double eta = (a + b - hAB) / 2;
    const double psum = 1.0 - pa - pb;
    double da = hAB * pb + eta - a;
    double db = hAB * pa + eta - b;
    da -= wcmp * psum;
    db -= wcmp * psum;
    wa[i] = a + wopt * da;
    wb[i] = b + wopt * db;
  });
}

// phi_w_constrained (cuda_aid.cu:418-452): simple mixing plus a penalty
// pulling phiA toward the target T with weight lambda; its constants are the
// reference's hard-coded wopt 0.05, wcmp 0.10.
__global__ void k_phi_w_constrained(double *__restrict__ wa, double *__restrict__ wb,
                                    const double *__restrict__ pha,
                                    const double *__restrict__ phb,
                                    const double *__restrict__ tgt, double hAB, double lambda,
                                    long long n) {
  const double wopt = 0.050, wcmp = 0.10;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double a = wa[i], b = wb[i], pa = pha[i], pb = phb[i], t = tgt[i];
    const double eta = (a + b - hAB) / 2;
    const double psum = 1.0 - pa - pb;
    double da = hAB * pb + eta - a + lambda * (pa - t);
    double db = hAB * pa + eta - b + lambda * (pb - (1 - t));
    da -= wcmp * psum;
    db -= wcmp * psum;
    wa[i] = a + wopt * da;
    wb[i] = b + wopt * db;
  }
}

// phi_w_constrainedEx (cuda_aid.cu:454-490): the exchange-field form with the
// reference's hard-coded wopt 1.60, wcmp 0.50.
__global__ void k_phi_w_constrained_ex(double *__restrict__ wa, double *__restrict__ wb,
                                       const double *__restrict__ pha,
                                       const double *__restrict__ phb,
                                       const double *__restrict__ tgt, double hAB, long long n) {
  const double wopt = 1.60, wcmp = 0.50;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double a = wa[i], b = wb[i], pa = pha[i], pb = phb[i], t = tgt[i];
    const double wum = -hAB * (t * 2 - 1) - (a - b);
    const double eta = (a + b - hAB + wum) / 2;
    const double psum = 1.0 - pa - pb;
    const double psum1 = pa - t;
    double da = hAB * (1 - t) + eta - a - wum;
    double db = hAB * t + eta - b;
    da -= 2.0 * wcmp * psum - 2.0 * wcmp * psum1;
    db -= 2 * wcmp * psum1;
    wa[i] = a + wopt * da;
    wb[i] = b + wopt * db;
  }
}

// Contour-outer propagator [b][s][M] (working precision) -> the reference's
// layout g[b][r][s] in FP64, s fastest (cuda_aid.cu:237), by 32x32 tiles
// through shared memory so both sides stay coalesced.
template <typename R>
__global__ void k_q_to_reference_layout(const R *__restrict__ q, int ns1, long long M,
                                        double *__restrict__ g) {
  __shared__ double tile[32][33];
  const long long b = blockIdx.z;
  const long long r0 = (long long)blockIdx.x * 32;
  const int s0 = blockIdx.y * 32;
  const R *qb = q + b * ns1 * M;
  double *gb = g + b * ns1 * M;
  for (int k = threadIdx.y; k < 32; k += 8) {
    const int s = s0 + k;
    const long long r = r0 + threadIdx.x;
    if (s < ns1 && r < M) tile[k][threadIdx.x] = (double)qb[(long long)s * M + r];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += 8) {
    const long long r = r0 + k;
    const int s = s0 + threadIdx.x;
    if (s < ns1 && r < M) gb[r * ns1 + s] = tile[threadIdx.x][k];
  }
}

// partial layout: [b][3][nblk]
__global__ void k_fe_partials(const double *__restrict__ wa, const double *__restrict__ wb,
                              const double *__restrict__ pha, const double *__restrict__ phb,
                              double hAB, long long M, double *__restrict__ partial) {
  __shared__ double sh[32];
  const long long o = blockIdx.y * M;
  double fab = 0.0, fw = 0.0, inc = 0.0;
  auto load = [&](long long i) { return dquad{wa[o + i], wb[o + i], pha[o + i], phb[o + i]}; };
  stream_loop<4>(M, load,
                 [&](long long, dquad v) {
    const double pa = v.z, pb = v.w;
    fab += hAB * pa * pb;                          // cuda_scft.cu:207
    fw += v.x * pa + v.y * pb;                     // cuda_scft.cu:208
    inc = fmax(inc, fabs(1.0 - pa - pb));          // cuda_scft.cu:203-206
  });
  const int nb = gridDim.x;
  double r;
  r = block_sum(fab, sh);
  if (threadIdx.x == 0) partial[(blockIdx.y * 3 + 0) * nb + blockIdx.x] = r;
  r = block_sum(fw, sh);
  if (threadIdx.x == 0) partial[(blockIdx.y * 3 + 1) * nb + blockIdx.x] = r;
  r = block_max(inc, sh);
  if (threadIdx.x == 0) partial[(blockIdx.y * 3 + 2) * nb + blockIdx.x] = r;
}

// out5[b] = {F, F_AB, F_W, F_S, inCompMax}
__global__ void k_fe_finalize(const double *__restrict__ partial, int nblk, long long M,
                              const double *__restrict__ Q, double *__restrict__ out5) {
  __shared__ double sh[32];
  const int b = blockIdx.x;
  double s0 = 0.0, s1 = 0.0, m2 = 0.0;
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) {
    s0 += partial[(b * 3 + 0) * nblk + i];
    s1 += partial[(b * 3 + 1) * nblk + i];
    m2 = fmax(m2, partial[(b * 3 + 2) * nblk + i]);
  }
  s0 = block_sum(s0, sh);
  s1 = block_sum(s1, sh);
  m2 = block_max(m2, sh);
  if (threadIdx.x == 0) {
    const double fab = s0 / (double)M, fw = -s1 / (double)M, fs = -log(Q[b]);
    out5[b * 5 + 0] = fab + fw + fs;   // cuda_scft.cu:220
    out5[b * 5 + 1] = fab;
    out5[b * 5 + 2] = fw;
    out5[b * 5 + 3] = fs;
    out5[b * 5 + 4] = m2;
  }
}

inline int grid_for(long long n) {
  long long g = (n + kThreads - 1) / kThreads;
  if (g > 152 * 16) g = 152 * 16;
  if (g < 1) g = 1;
  return (int)g;
}

}  // namespace

int reduce_blocks(long long M) {
  long long g = (M + kThreads * 4 - 1) / (kThreads * 4);
  if (g > 152 * 4) g = 152 * 4;
  if (g < 1) g = 1;
  return (int)g;
}

template <typename R>
cudaError_t launch_boltzmann(const double *w, R *W, long long n, double ds2, cudaStream_t st) {
  k_boltzmann<R><<<grid_for(n), kThreads, 0, st>>>(w, W, n, ds2);
  return cudaGetLastError();
}
template <typename R>
cudaError_t launch_fill(R *x, long long n, R v, long long bstride, int batch, cudaStream_t st) {
  k_fill<R><<<dim3(grid_for(n), batch), kThreads, 0, st>>>(x, n, v, bstride);
  return cudaGetLastError();
}
template <typename R>
cudaError_t launch_copy_slice(R *dst, long long dbs, const R *src, long long sbs, long long M,
                              int batch, cudaStream_t st) {
  k_copy<R, R><<<dim3(grid_for(M), batch), kThreads, 0, st>>>(dst, dbs, src, sbs, M);
  return cudaGetLastError();
}
template <typename R>
cudaError_t launch_cast_slice(double *dst, long long dbs, const R *src, long long sbs,
                              long long M, int batch, cudaStream_t st) {
  k_copy<R, double><<<dim3(grid_for(M), batch), kThreads, 0, st>>>(dst, dbs, src, sbs, M);
  return cudaGetLastError();
}
template <typename R>
cudaError_t launch_partial_sum(const R *x, long long bs, long long M, int batch, double *partial,
                               int nblk, cudaStream_t st) {
  k_partial_sum<R><<<dim3(nblk, batch), kThreads, 0, st>>>(x, bs, M, partial);
  return cudaGetLastError();
}
cudaError_t launch_finalize_sum(const double *partial, int nblk, int batch, double scale,
                                double *out, cudaStream_t st) {
  k_finalize_sum<<<batch, kThreads, 0, st>>>(partial, nblk, scale, out);
  return cudaGetLastError();
}
cudaError_t launch_minus_average(double *data, const double *sum, long long M, int batch,
                                 cudaStream_t st) {
  k_minus_average<<<dim3(grid_for(M), batch), kThreads, 0, st>>>(data, sum, M);
  return cudaGetLastError();
}
cudaError_t launch_q_ffl(const double *sum, long long M, double ds0, int batch, double *Q,
                         double *ffl, cudaStream_t st) {
  k_q_ffl<<<(batch + 127) / 128, 128, 0, st>>>(sum, M, ds0, batch, Q, ffl);
  return cudaGetLastError();
}
double contour_weight(int s, int n, bool simpson) {
  if (s < 0 || s > n) return 0.0;
  if (n == 0) return 0.5;                                 // cuda_aid.cu:91
  if (!simpson || n == 1) return (s == 0 || s == n) ? 0.5 : 1.0;
  const int m = (n % 2 == 0) ? n : n - 3;                 // end of the 1/3 rule
  double w = 0.0;
  if (m > 0 && s <= m) w += (s == 0 || s == m) ? 1.0 / 3.0 : ((s & 1) ? 4.0 / 3.0 : 2.0 / 3.0);
  if (m < n && s >= m) w += (s == m || s == n) ? 3.0 / 8.0 : 9.0 / 8.0;   // the 3/8 rule
  return w;
}

ContourWeights contour_weights(int n, bool simpson) {
  ContourWeights cw;
  memset(&cw, 0, sizeof cw);
  cw.c_odd = cw.c_even = 1.0;
  if (n == 0) {
    cw.m = 0;
    cw.nspec = 1;
    cw.s[0] = 0;
    cw.w[0] = 0.5;
    return cw;
  }
  if (!simpson || n == 1) {
    cw.m = n;
    cw.nspec = 2;
    cw.s[0] = 0; cw.w[0] = 0.5;
    cw.s[1] = n; cw.w[1] = 0.5;
    return cw;
  }
  const int m = (n % 2 == 0) ? n : n - 3;
  cw.c_odd = 4.0 / 3.0;
  cw.c_even = 2.0 / 3.0;
  cw.m = m > 0 ? m : 1;                                   // interior 1..m-1
  int k = 0;
  for (int s = 0; s <= n; ++s) {
    const bool interior = s >= 1 && s < cw.m;
    if (!interior) {
      cw.s[k] = s;
      cw.w[k] = contour_weight(s, n, true);
      ++k;
    }
  }
  cw.nspec = k;
  return cw;
}

template <typename R>
cudaError_t launch_contour_phi(const R *q, const R *qc, int ns, long long M, int batch,
                               const double *ffl, double *phi, bool simpson, cudaStream_t st) {
  const ContourWeights cw = contour_weights(ns, simpson);
  if (cw.nspec > 5) return cudaErrorInvalidValue;
  k_contour_phi<R><<<dim3(grid_for(M), batch), kThreads, 0, st>>>(q, qc, ns, M, ffl, phi, cw);
  return cudaGetLastError();
}
cudaError_t launch_phi_w(double *wa, double *wb, const double *pha, const double *phb,
                         double hAB, double wopt, double wcmp, long long M, int batch,
                         cudaStream_t st) {
  const long long n = M * batch;
  k_phi_w<<<grid_for(n), kThreads, 0, st>>>(wa, wb, pha, phb, hAB, wopt, wcmp, n);
  return cudaGetLastError();
}
template <typename R>
cudaError_t launch_q_to_reference_layout(const R *q, int ns, long long M, int batch, double *g,
                                         cudaStream_t st) {
  const long long gx = (M + 31) / 32;
  if (gx > 0x7fffffffLL || batch > 65535) return cudaErrorInvalidValue;
  dim3 grid((unsigned)gx, (unsigned)((ns + 1 + 31) / 32), batch);
  k_q_to_reference_layout<R><<<grid, dim3(32, 8), 0, st>>>(q, ns + 1, M, g);
  return cudaGetLastError();
}
template cudaError_t launch_q_to_reference_layout<float>(const float *, int, long long, int,
                                                         double *, cudaStream_t);
template cudaError_t launch_q_to_reference_layout<double>(const double *, int, long long, int,
                                                          double *, cudaStream_t);
template cudaError_t launch_q_to_reference_layout<dfloat>(const dfloat *, int, long long, int,
                                                          double *, cudaStream_t);

cudaError_t launch_phi_w_constrained(double *wa, double *wb, const double *pha, const double *phb,
                                     const double *target, double hAB, double lambda, int ex,
                                     long long M, int batch, cudaStream_t st) {
  const long long n = M * batch;
  if (ex)
    k_phi_w_constrained_ex<<<grid_for(n), kThreads, 0, st>>>(wa, wb, pha, phb, target, hAB, n);
  else
    k_phi_w_constrained<<<grid_for(n), kThreads, 0, st>>>(wa, wb, pha, phb, target, hAB, lambda,
                                                           n);
  return cudaGetLastError();
}

cudaError_t launch_free_energy_partials(const double *wa, const double *wb, const double *pha,
                                        const double *phb, double hAB, long long M, int batch,
                                        double *partial, int nblk, cudaStream_t st) {
  k_fe_partials<<<dim3(nblk, batch), kThreads, 0, st>>>(wa, wb, pha, phb, hAB, M, partial);
  return cudaGetLastError();
}
cudaError_t launch_free_energy_finalize(const double *partial, int nblk, int batch, long long M,
                                        const double *Q, double *out5, cudaStream_t st) {
  k_fe_finalize<<<batch, kThreads, 0, st>>>(partial, nblk, M, Q, out5);
  return cudaGetLastError();
}

#define INST(R)                                                                                  \
  template cudaError_t launch_boltzmann<R>(const double *, R *, long long, double, cudaStream_t); \
  template cudaError_t launch_fill<R>(R *, long long, R, long long, int, cudaStream_t);           \
  template cudaError_t launch_copy_slice<R>(R *, long long, const R *, long long, long long, int, \
                                            cudaStream_t);                                        \
  template cudaError_t launch_cast_slice<R>(double *, long long, const R *, long long, long long, \
                                            int, cudaStream_t);                                   \
  template cudaError_t launch_partial_sum<R>(const R *, long long, long long, int, double *, int, \
                                             cudaStream_t);                                       \
  template cudaError_t launch_contour_phi<R>(const R *, const R *, int, long long, int,           \
                                             const double *, double *, bool, cudaStream_t);
INST(float)
INST(double)
INST(dfloat)
#undef INST

}  // namespace scft
