// Field-update kernels with a convergence measure: simple mixing with its
// residual, and Anderson mixing (no reference counterpart; the reference has
// only phi_w, cuda_aid.cu:382-416).
//
// Residual (phi_w's update direction before the wopt step, cuda_aid.cu:398-408):
//   dA = hAB*phB + eta - wA - wcmp*(1-phA-phB),  dB = hAB*phA + eta - wB - wcmp*(...)
// Anderson (Anderson 1965, in the form used for SCFT by Thompson et al. 2004 and
// Matsen 2009): keep the last m+1 iterations in a ring; with G_ij = <d_i, d_j>
// (both fields, all points) and the current slot c,
//   U_ij = G_cc - G_c,ci - G_c,cj + G_ci,cj ,  V_i = G_cc - G_c,ci   (ci = slot c-i)
//   solve U x = V (FP64, one warp);  a_c = 1 - sum x_i, a_ci = x_i
//   w_new = sum_j a_j (w_j + lambda d_j) = sum_j a_j u_j
// The ring holds u_j = w_j + lambda d_j (what the update reads) and d_j (what
// the Gram row reads), each as double-float pairs (hi, lo floats, about 48
// significant bits, dfloat.cuh): the Gram row and the update are sums of
// products over all slots and points, which on GB300's FP64 pipe took 3x
// their memory time; in pair arithmetic on the FP32 pipe they run at the
// speed of their loads, and storing u instead of (w, d) halves the update's.
// The Gram matrix, the solve and the fields stay FP64.
// An instance whose max|d| is still above `start` (or with no history yet)
// takes the simple step w_new = w_c + wopt d_c, decided on the device.
#include "common.cuh"
#include "dfloat.cuh"
#include "kernels.h"

namespace scft {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ double blk_sum(double v, double *sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (wid == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    r = warp_sum(r);
  }
  return r;
}
__device__ __forceinline__ double blk_max(double v, double *sh) {
  v = warp_max(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (wid == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    r = warp_max(r);
  }
  return r;
}

// |x| as an ordered integer key: for non-negative doubles the unsigned bit
// patterns order like the values, and a NaN (sign cleared) sorts above +inf,
// so a maximum over keys propagates NaN where fmax would drop it (a diverged
// field then reports a NaN residual instead of a finite one).
__device__ __forceinline__ unsigned long long abs_key(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
}
__device__ __forceinline__ unsigned long long key_max(unsigned long long a, unsigned long long b) {
  return a > b ? a : b;
}
__device__ __forceinline__ unsigned long long blk_max_key(unsigned long long v,
                                                          unsigned long long *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = key_max(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  unsigned long long r = 0;
  if (wid == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0ULL;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r = key_max(r, __shfl_xor_sync(0xffffffffu, r, o));
  }
  return r;
}

// phi_w's update direction (cuda_aid.cu:398-408).  It is affine in
// (wA, wB, phiA, phiB), so the instance mean of the direction is the
// direction of the instance means.
__device__ __forceinline__ void phi_w_dir(double a, double c, double pa, double pb, double hAB,
                                          double wcmp, double &da, double &db) {
  const double eta = (a + c - hAB) / 2;
  const double psum = 1.0 - pa - pb;
  da = hAB * pb + eta - a;
  db = hAB * pa + eta - c;
  da -= wcmp * psum;
  db -= wcmp * psum;
}

// Per-instance sums of wA, wB, phiA, phiB: partial[(b*4 + f)*nblk + blk].
// (Four additions per point: GB300's FP64 pipe, not HBM, bounds the
// per-point direction, so its mean is formed from these sums instead.)
__global__ void k_residual_sum(const double *__restrict__ wa, const double *__restrict__ wb,
                               const double *__restrict__ pha, const double *__restrict__ phb,
                               long long M, double *__restrict__ partial) {
  __shared__ double sh[32];
  const long long b = blockIdx.y, o = b * M;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  auto load = [&](long long i) { return dquad{wa[o + i], wb[o + i], pha[o + i], phb[o + i]}; };
  stream_loop<4>(M, load, [&](long long, dquad v) {
    s0 += v.x;
    s1 += v.y;
    s2 += v.z;
    s3 += v.w;
  });
  const double r[4] = {blk_sum(s0, sh), blk_sum(s1, sh), blk_sum(s2, sh), blk_sum(s3, sh)};
  if (threadIdx.x == 0)
    for (int f = 0; f < 4; ++f) partial[(b * 4 + f) * gridDim.x + blockIdx.x] = r[f];
}

// dmean[b*2 + f] = mean of dA / dB = the direction of the field means
__global__ void k_residual_mean(const double *__restrict__ partial, int nblk, long long M,
                                double hAB, double wcmp, double *__restrict__ dmean) {
  __shared__ double sh[32];
  const int b = blockIdx.x;
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < nblk; i += blockDim.x)
    for (int f = 0; f < 4; ++f) s[f] += partial[(b * 4 + f) * nblk + i];
  for (int f = 0; f < 4; ++f) s[f] = blk_sum(s[f], sh);
  if (threadIdx.x == 0) {
    const double m = (double)M;
    phi_w_dir(s[0] / m, s[1] / m, s[2] / m, s[3] / m, hAB, wcmp, dmean[b * 2 + 0],
              dmean[b * 2 + 1]);
  }
}

// Residual of instance blockIdx.y.  The field mean is a gauge freedom
// (average_value removes it every iteration), so the residual that measures
// convergence and enters the Anderson history is d = dir - mean(dir); the
// simple step applies the raw phi_w direction, exactly as the reference.
// Optionally stores u = w + lam_u d and d into a history slot ([b][2][M]
// double-float pairs), copies w to wprev ([b][2][M] FP64) and applies the
// simple step in place (wopt != 0).
// partial[(b*2 + {0: max|d|, 1: sum d^2})*nblk + blk]
__global__ void k_residual(double *__restrict__ wa, double *__restrict__ wb,
                           const double *__restrict__ pha, const double *__restrict__ phb,
                           double hAB, double wcmp, double wopt, long long M,
                           const double *__restrict__ dmean, dfloat *__restrict__ hu,
                           dfloat *__restrict__ hd, double lam_u, double *__restrict__ wprev,
                           double *__restrict__ partial) {
  __shared__ double sh[32];
  __shared__ unsigned long long shk[32];
  const long long b = blockIdx.y, o = b * M;
  const double ma = dmean[b * 2 + 0], mb = dmean[b * 2 + 1];
  unsigned long long mx = 0;
  double ss = 0.0;
  auto load = [&](long long i) { return dquad{wa[o + i], wb[o + i], pha[o + i], phb[o + i]}; };
  stream_loop<4>(M, load,
                 [&](long long i, dquad v) {
    const double a = v.x, c = v.y;
    double da, db;
    phi_w_dir(a, c, v.z, v.w, hAB, wcmp, da, db);   // cuda_aid.cu:398-408
    const double ca = da - ma, cb = db - mb;
    mx = key_max(mx, key_max(abs_key(ca), abs_key(cb)));
    ss += ca * ca + cb * cb;
    if (hu) {
      hu[(2 * b) * M + i] = dfloat(fma(lam_u, ca, a));
      hu[(2 * b + 1) * M + i] = dfloat(fma(lam_u, cb, c));
      hd[(2 * b) * M + i] = dfloat(ca);
      hd[(2 * b + 1) * M + i] = dfloat(cb);
    }
    if (wprev) {
      wprev[(2 * b) * M + i] = a;
      wprev[(2 * b + 1) * M + i] = c;
    }
    if (wopt != 0.0) {
      wa[o + i] = a + wopt * da;   // phi_w, cuda_aid.cu:410-412
      wb[o + i] = c + wopt * db;
    }
  });
  const unsigned long long rm = blk_max_key(mx, shk);
  const double rs = blk_sum(ss, sh);
  if (threadIdx.x == 0) {
    partial[(b * 2 + 0) * gridDim.x + blockIdx.x] = __longlong_as_double((long long)rm);
    partial[(b * 2 + 1) * gridDim.x + blockIdx.x] = rs;
  }
}

// err[b*2 + 0] = max|d|, err[b*2 + 1] = rms
__global__ void k_residual_finalize(const double *__restrict__ partial, int nblk, long long M,
                                    double *__restrict__ err) {
  __shared__ double sh[32];
  __shared__ unsigned long long shk[32];
  const int b = blockIdx.x;
  unsigned long long mx = 0;
  double ss = 0.0;
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) {
    mx = key_max(mx, abs_key(partial[(b * 2 + 0) * nblk + i]));
    ss += partial[(b * 2 + 1) * nblk + i];
  }
  mx = blk_max_key(mx, shk);
  ss = blk_sum(ss, sh);
  if (threadIdx.x == 0) {
    err[b * 2 + 0] = __longlong_as_double((long long)mx);
    err[b * 2 + 1] = sqrt(ss / (2.0 * (double)M));
  }
}

// acc += x * y in pair arithmetic, the product's error term left
// unnormalised (it only enters the sum's low part).
__device__ __forceinline__ void df_fma_acc(dfloat &acc, dfloat x, dfloat y) {
  const float p = x.hi * y.hi;
  float e = fmaf(x.hi, y.hi, -p);
  e = fmaf(x.hi, y.lo, e);
  e = fmaf(x.lo, y.hi, e);
  const dfloat s = df_two_sum(acc.hi, p);
  acc = df_fast_two_sum(s.hi, s.lo + (acc.lo + e));
}
__device__ __forceinline__ dfloat ld_pair(const dfloat *p) {
  const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
  return dfloat(v.x, v.y);
}

// Gram row of slot c: <d_c, d_j> for the listed slots j (nj <= kMaxSlots).
// partial[(b*kMaxSlots + k)*nblk + blk]
constexpr int kMaxSlots = 33;
struct SlotList {
  const dfloat *d[kMaxSlots];
  int slot[kMaxSlots];
  int n;
};
// Grid row blockIdx.y takes the kChunk list entries from blockIdx.y*kChunk:
// few accumulators keep the occupancy high and each thread has kChunk + 1
// loads in flight per element; d_c is read once per chunk (an L2 hit while
// it fits).
constexpr int kChunk = 8;
__global__ void k_gram_row(const dfloat *__restrict__ dc, SlotList sl, long long M,
                           double *__restrict__ partial) {
  __shared__ double sh[32];
  const long long b = blockIdx.z;
  const int k0 = blockIdx.y * kChunk;
  const long long n2 = 2 * M;
  const dfloat *dk[kChunk];
  dfloat acc[kChunk];
#pragma unroll
  for (int kk = 0; kk < kChunk; ++kk)
    dk[kk] = k0 + kk < sl.n ? sl.d[k0 + kk] + b * n2 : nullptr;
  const dfloat *x = dc + b * n2;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n2;
       i += (long long)gridDim.x * blockDim.x) {
    dfloat y[kChunk];
#pragma unroll
    for (int kk = 0; kk < kChunk; ++kk)
      if (dk[kk]) y[kk] = ld_pair(dk[kk] + i);
    const dfloat xi = ld_pair(x + i);
#pragma unroll
    for (int kk = 0; kk < kChunk; ++kk)
      if (dk[kk]) df_fma_acc(acc[kk], xi, y[kk]);
  }
#pragma unroll
  for (int kk = 0; kk < kChunk; ++kk) {
    if (dk[kk]) {
      const double r = blk_sum((double)acc[kk], sh);
      if (threadIdx.x == 0)
        partial[(b * kMaxSlots + k0 + kk) * gridDim.x + blockIdx.x] = r;
    }
  }
}

// Finalise the Gram row into the ring matrix G[b][(m+1)x(m+1)] (symmetric).
__global__ void k_gram_finalize(const double *__restrict__ partial, int nblk, SlotList sl, int c,
                                int m1, double *__restrict__ G) {
  __shared__ double sh[32];
  const int b = blockIdx.y, k = blockIdx.x;
  if (k >= sl.n) return;
  double s = 0.0;
  for (int i = threadIdx.x; i < nblk; i += blockDim.x)
    s += partial[((long long)b * kMaxSlots + k) * nblk + i];
  s = blk_sum(s, sh);
  if (threadIdx.x == 0) {
    const int j = sl.slot[k];
    G[((long long)b * m1 + c) * m1 + j] = s;
    G[((long long)b * m1 + j) * m1 + c] = s;
  }
}

// One warp per instance: weights a[b][slot] and the step lam_eff[b].
// hist = number of previous slots (newest first: c-1, c-2, ...).
// mode[b] = 1 for an Anderson step, 0 for the simple step.
__global__ void k_anderson_solve(const double *__restrict__ G, const double *__restrict__ err,
                                 int c, int hist, int m1, double start, double lambda,
                                 double wopt, double *__restrict__ a, double *__restrict__ lam,
                                 double *__restrict__ mode) {
  __shared__ double U[32][33];
  __shared__ double V[32];
  const int b = blockIdx.x, lane = threadIdx.x;
  const double *Gb = G + (long long)b * m1 * m1;
  double *ab = a + (long long)b * m1;
  for (int j = lane; j < m1; j += 32) ab[j] = 0.0;
  __syncwarp();
  const bool simple = hist == 0 || !(err[b * 2] < start);
  if (simple) {
    if (lane == 0) {
      ab[c] = 1.0;
      lam[b] = wopt;
      mode[b] = 0.0;
    }
    return;
  }
  const int n = hist;
  auto slot = [&](int i) { return ((c - i) % m1 + m1) % m1; };   // i = 1..n
  const double gcc = Gb[c * m1 + c];
  for (int i = 0; i < n; ++i) {
    if (lane < n) {
      const int si = slot(i + 1), sj = slot(lane + 1);
      U[i][lane] = gcc - Gb[c * m1 + si] - Gb[c * m1 + sj] + Gb[si * m1 + sj];
    }
  }
  if (lane < n) V[lane] = gcc - Gb[c * m1 + slot(lane + 1)];
  __syncwarp();
  // Tikhonov shift relative to the largest diagonal entry keeps U invertible
  // when two histories are nearly parallel.
  double dmax = 0.0;
  for (int i = 0; i < n; ++i) dmax = fmax(dmax, fabs(U[i][i]));
  if (lane < n) U[lane][lane] += 1e-12 * dmax + 1e-300;
  __syncwarp();
  // Gaussian elimination with partial pivoting; lane r owns row r.
  for (int k = 0; k < n; ++k) {
    int piv = k;
    if (lane == 0) {
      double best = fabs(U[k][k]);
      for (int r = k + 1; r < n; ++r)
        if (fabs(U[r][k]) > best) { best = fabs(U[r][k]); piv = r; }
    }
    piv = __shfl_sync(0xffffffffu, piv, 0);
    if (piv != k) {
      if (lane <= n) {
        if (lane < n) {
          const double t = U[k][lane]; U[k][lane] = U[piv][lane]; U[piv][lane] = t;
        }
      }
      if (lane == 0) { const double t = V[k]; V[k] = V[piv]; V[piv] = t; }
    }
    __syncwarp();
    const double pk = U[k][k];
    if (lane > k && lane < n) {
      const double f = U[lane][k] / pk;
      for (int j = k; j < n; ++j) U[lane][j] -= f * U[k][j];
      V[lane] -= f * V[k];
    }
    __syncwarp();
  }
  if (lane == 0) {
    double x[32];
    double sx = 0.0;
    for (int i = n - 1; i >= 0; --i) {
      double s = V[i];
      for (int j = i + 1; j < n; ++j) s -= U[i][j] * x[j];
      x[i] = s / U[i][i];
    }
    for (int i = 0; i < n; ++i) {
      ab[slot(i + 1)] = x[i];
      sx += x[i];
    }
    ab[c] = 1.0 - sx;
    lam[b] = lambda;
    mode[b] = 1.0;
  }
}

// Anderson step: w_new = sum_j a_j u_j over the listed slots, in pair
// arithmetic; simple step (mode 0): w_new = w + lam d_c in FP64 from the live
// fields.  kUChunk slots' loads are in flight per element.
struct SlotRing {
  const dfloat *u[kMaxSlots];
  int idx[kMaxSlots];
  int n;
};
constexpr int kUChunk = 8;
__global__ void k_anderson_update(double *__restrict__ wa, double *__restrict__ wb, SlotRing sr,
                                  const dfloat *__restrict__ dc, const double *__restrict__ a,
                                  const double *__restrict__ lam, const double *__restrict__ mode,
                                  int m1, long long M) {
  __shared__ dfloat s_a[kMaxSlots];   // the weights of the listed slots
  const long long b = blockIdx.y;
  const long long n2 = 2 * M;
  const long long S = (long long)gridDim.x * blockDim.x;
  double *wab = wa + b * M, *wbb = wb + b * M;
  if (mode[b] == 0.0) {
    const double l = lam[b];
    const dfloat *d = dc + b * n2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n2; i += S) {
      double *w = i < M ? wab + i : wbb + (i - M);
      *w = fma(l, (double)ld_pair(d + i), *w);
    }
    return;
  }
  for (int k = threadIdx.x; k < sr.n; k += blockDim.x) s_a[k] = dfloat(a[b * m1 + sr.idx[k]]);
  __syncthreads();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n2; i += S) {
    dfloat s;
    for (int k0 = 0; k0 < sr.n; k0 += kUChunk) {
      dfloat y[kUChunk];
#pragma unroll
      for (int kk = 0; kk < kUChunk; ++kk)
        if (k0 + kk < sr.n) y[kk] = ld_pair(sr.u[k0 + kk] + b * n2 + i);
#pragma unroll
      for (int kk = 0; kk < kUChunk; ++kk)
        if (k0 + kk < sr.n) df_fma_acc(s, s_a[k0 + kk], y[kk]);
    }
    if (i < M) wab[i] = (double)s;
    else wbb[i - M] = (double)s;
  }
}

// ---- the update without its rigid-shift component (SCFT_FLAG_PIN_TRANSLATION)
// Rigid-shift generators of the pre-update fields w0 ([b][2][M], the Anderson
// ring slot of this iteration): central differences along each axis longer
// than one point, periodic, in grid units.
struct Grid3 {
  int nx, ny, nz;
};
__device__ __forceinline__ void shift_gen(const double *__restrict__ w0, long long i, Grid3 g,
                                          double t[3]) {
  const long long nxy = (long long)g.nx * g.ny;
  const int x = (int)(i % g.nx), y = (int)((i / g.nx) % g.ny), z = (int)(i / nxy);
  const long long row = i - x, col = i - (long long)y * g.nx, pln = i - (long long)z * nxy;
  t[0] = g.nx > 1 ? 0.5 * (w0[row + (x + 1) % g.nx] - w0[row + (x + g.nx - 1) % g.nx]) : 0.0;
  t[1] = g.ny > 1 ? 0.5 * (w0[col + (long long)((y + 1) % g.ny) * g.nx] -
                           w0[col + (long long)((y + g.ny - 1) % g.ny) * g.nx])
                  : 0.0;
  t[2] = g.nz > 1 ? 0.5 * (w0[pln + (long long)((z + 1) % g.nz) * nxy] -
                           w0[pln + (long long)((z + g.nz - 1) % g.nz) * nxy])
                  : 0.0;
}

// Per instance and block: the six Gram entries <t_a, t_b> and the three
// projections <t_a, w1 - w0>, over both fields.
// partial[(b*9 + k)*nblk + blk], k: G00 G01 G02 G11 G12 G22 c0 c1 c2
__global__ void k_shift_dots(const double *__restrict__ wa1, const double *__restrict__ wb1,
                             const double *__restrict__ w0, long long M, Grid3 g,
                             double *__restrict__ partial) {
  __shared__ double sh[32];
  const long long b = blockIdx.y;
  double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < M;
       i += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int f = 0; f < 2; ++f) {
      const double *w0f = w0 + (2 * b + f) * M;
      double t[3];
      shift_gen(w0f, i, g, t);
      const double d = (f ? wb1 : wa1)[b * M + i] - w0f[i];
      acc[0] += t[0] * t[0];
      acc[1] += t[0] * t[1];
      acc[2] += t[0] * t[2];
      acc[3] += t[1] * t[1];
      acc[4] += t[1] * t[2];
      acc[5] += t[2] * t[2];
      acc[6] += t[0] * d;
      acc[7] += t[1] * d;
      acc[8] += t[2] * d;
    }
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const double r = blk_sum(acc[k], sh);
    if (threadIdx.x == 0) partial[(b * 9 + k) * gridDim.x + blockIdx.x] = r;
  }
}

// alpha[b*3 + a]: least-squares shift coefficients over the axes longer than
// one point (the normal equations with a 1e-14 relative diagonal shift).
__global__ void k_shift_solve(const double *__restrict__ partial, int nblk, Grid3 g,
                              double *__restrict__ alpha) {
  __shared__ double sh[32];
  const int b = blockIdx.x;
  double s[9];
  for (int k = 0; k < 9; ++k) {
    double v = 0.0;
    for (int i = threadIdx.x; i < nblk; i += blockDim.x) v += partial[(b * 9 + k) * nblk + i];
    s[k] = blk_sum(v, sh);
  }
  if (threadIdx.x != 0) return;
  const double G[3][3] = {{s[0], s[1], s[2]}, {s[1], s[3], s[4]}, {s[2], s[4], s[5]}};
  const int n3[3] = {g.nx, g.ny, g.nz};
  int ax[3], n = 0;
  for (int a = 0; a < 3; ++a)
    if (n3[a] > 1) ax[n++] = a;
  double A[3][4], dmax = 0.0;
  for (int i = 0; i < n; ++i) dmax = fmax(dmax, fabs(G[ax[i]][ax[i]]));
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < n; ++j) A[i][j] = G[ax[i]][ax[j]];
    A[i][i] += 1e-14 * dmax + 1e-300;
    A[i][3] = s[6 + ax[i]];
  }
  // Gaussian elimination (symmetric positive definite: no pivoting needed)
  for (int k = 0; k < n; ++k)
    for (int r = k + 1; r < n; ++r) {
      const double f = A[r][k] / A[k][k];
      for (int j = k; j < 4; ++j) A[r][j] -= f * A[k][j];
    }
  double x[3] = {0.0, 0.0, 0.0};
  for (int i = n - 1; i >= 0; --i) {
    double v = A[i][3];
    for (int j = i + 1; j < n; ++j) v -= A[i][j] * x[j];
    x[i] = v / A[i][i];
  }
  double out[3] = {0.0, 0.0, 0.0};
  for (int i = 0; i < n; ++i) out[ax[i]] = x[i];
  for (int a = 0; a < 3; ++a) alpha[b * 3 + a] = out[a];
}

// w1 -= sum_a alpha_a t_a(w0), both fields
__global__ void k_shift_apply(double *__restrict__ wa1, double *__restrict__ wb1,
                              const double *__restrict__ w0, long long M, Grid3 g,
                              const double *__restrict__ alpha) {
  const long long b = blockIdx.y;
  const double a0 = alpha[b * 3], a1 = alpha[b * 3 + 1], a2 = alpha[b * 3 + 2];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < M;
       i += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int f = 0; f < 2; ++f) {
      double t[3];
      shift_gen(w0 + (2 * b + f) * M, i, g, t);
      double *w1 = (f ? wb1 : wa1) + b * M;
      w1[i] -= a0 * t[0] + a1 * t[1] + a2 * t[2];
    }
  }
}

inline int grid_for(long long n) {
  long long g = (n + kThreads - 1) / kThreads;
  if (g > 152 * 8) g = 152 * 8;
  return g < 1 ? 1 : (int)g;
}

}  // namespace

int anderson_max_slots() { return kMaxSlots; }

cudaError_t launch_residual(double *wa, double *wb, const double *pha, const double *phb,
                            double hAB, double wcmp, double wopt, long long M, int batch,
                            void *hu, void *hd, double lam_u, double *wprev, double *partial,
                            int nblk, double *err, cudaStream_t st) {
  // err holds [b][2] results; err + 2*batch holds the [b][2] means of dA, dB
  double *dmean = err + 2 * batch;
  k_residual_sum<<<dim3(nblk, batch), kThreads, 0, st>>>(wa, wb, pha, phb, M, partial);
  k_residual_mean<<<batch, kThreads, 0, st>>>(partial, nblk, M, hAB, wcmp, dmean);
  k_residual<<<dim3(nblk, batch), kThreads, 0, st>>>(
      wa, wb, pha, phb, hAB, wcmp, wopt, M, dmean, static_cast<dfloat *>(hu),
      static_cast<dfloat *>(hd), lam_u, wprev, partial);
  k_residual_finalize<<<batch, kThreads, 0, st>>>(partial, nblk, M, err);
  return cudaGetLastError();
}

cudaError_t launch_gram_row(const void *dc, const void *const *dj, const int *slots, int n,
                            int c, int m1, long long M, int batch, double *partial, int nblk,
                            double *G, cudaStream_t st) {
  if (n < 1 || n > kMaxSlots) return cudaErrorInvalidValue;
  SlotList sl;
  sl.n = n;
  for (int k = 0; k < n; ++k) {
    sl.d[k] = static_cast<const dfloat *>(dj[k]);
    sl.slot[k] = slots[k];
  }
  k_gram_row<<<dim3(nblk, (n + kChunk - 1) / kChunk, batch), kThreads, 0, st>>>(
      static_cast<const dfloat *>(dc), sl, M, partial);
  k_gram_finalize<<<dim3(n, batch), kThreads, 0, st>>>(partial, nblk, sl, c, m1, G);
  return cudaGetLastError();
}

cudaError_t launch_anderson_solve(const double *G, const double *err, int c, int hist, int m1,
                                  double start, double lambda, double wopt, int batch,
                                  double *a, double *lam, cudaStream_t st) {
  k_anderson_solve<<<batch, 32, 0, st>>>(G, err, c, hist, m1, start, lambda, wopt, a, lam,
                                         lam + batch);
  return cudaGetLastError();
}

cudaError_t launch_remove_translation(double *wa, double *wb, const double *w0, int nx, int ny,
                                     int nz, int batch, double *partial, int nblk,
                                     double *alpha, cudaStream_t st) {
  const Grid3 g{nx, ny, nz};
  const long long M = (long long)nx * ny * nz;
  k_shift_dots<<<dim3(nblk, batch), kThreads, 0, st>>>(wa, wb, w0, M, g, partial);
  k_shift_solve<<<batch, kThreads, 0, st>>>(partial, nblk, g, alpha);
  k_shift_apply<<<dim3(grid_for(M), batch), kThreads, 0, st>>>(wa, wb, w0, M, g, alpha);
  return cudaGetLastError();
}

cudaError_t launch_anderson_update(double *wa, double *wb, const void *const *hu, const void *dc,
                                   const int *idx, int n, const double *a, const double *lam,
                                   int m1, long long M, int batch, cudaStream_t st) {
  if (n < 1 || n > kMaxSlots) return cudaErrorInvalidValue;
  SlotRing sr;
  sr.n = n;
  for (int k = 0; k < n; ++k) {
    sr.u[k] = static_cast<const dfloat *>(hu[k]);
    sr.idx[k] = idx[k];
  }
  k_anderson_update<<<dim3(grid_for(2 * M), batch), kThreads, 0, st>>>(
      wa, wb, sr, static_cast<const dfloat *>(dc), a, lam, lam + batch, m1, M);
  return cudaGetLastError();
}

}  // namespace scft
