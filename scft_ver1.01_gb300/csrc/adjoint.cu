// Derivatives of getConc (cuda_scft.cu:61-138): the box stress from the
// stored propagators, and the reverse-mode adjoint of the whole propagator
// march with contour checkpointing.  The reference has neither.
//
// Notation.  The two propagator chains of getConc form one chain of
// N = NsA + dNsB steps: q(0) = 1, q(s) = A_s q(s-1) (qA then qB), and the
// complementary chain q+(N) = 1, q+(s-1) = A_s q+(s) (q+B then q+A), with the
// split step A_s = W K W, W = exp(-w ds/2) of the block's field and K the
// diffusion filter exp(-ds k^2).  K is real, even and circulant, so A_s is
// symmetric and its adjoint is A_s itself.  Q = <q(N)>,
// phiA/B = (ds/Q) * contour sums (trapezoid or Simpson weights) of q q+ over
// the block's contour points.
//
// Box derivative of one step: dA_s/dL_a = W (dK/dL_a) W, where dK/dL_a is K
// with the axis-a gain multiplied by 2 ds k_a^2 / L_a (k_a ~ 1/L_a), or, for
// a length-1 axis (whose k is the constant 2 pi / L), the whole K times that
// factor.  Hence dQ/dL_a = (1/M) sum_s <q+(s), W (dK/dL_a) W q(s-1)>.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "common.cuh"
#include "ctx.h"

#define CK(call)                                                                        \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return scft_fail(ctx, SCFT_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define CKL(call)                                                                       \
  do {                                                                                  \
    ++ctx->launches;                                                                    \
    CK(call);                                                                           \
  } while (0)

#define RC(call)                                                                        \
  do {                                                                                  \
    int rc_ = (call);                                                                   \
    if (rc_) return rc_;                                                                \
  } while (0)

namespace {

using scft::warp_sum;
constexpr int kT = 256;

int grid_for(long long n) {
  long long g = (n + kT - 1) / kT;
  return (int)std::min<long long>(g, 1 << 20);
}

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
  return r;
}

// acc1[b*nblk + blk] += sum_{j<cnt, r} a[b,j,r] * c1[b,j,r]  (and acc2 with c2)
// Slices j are M apart; every (b, blk) slot has one writer, so repeated
// calls accumulate in a fixed order (bit-reproducible).
template <typename R, typename S>
__global__ void k_dot_acc(const R *__restrict__ a, long long a_bs, const S *__restrict__ c1,
                          long long c1_bs, const S *__restrict__ c2, long long c2_bs,
                          long long M, int cnt, double *__restrict__ acc1,
                          double *__restrict__ acc2) {
  __shared__ double sh[32];
  const long long b = blockIdx.y;
  const int nblk = gridDim.x;
  double v1 = 0.0, v2 = 0.0;
  for (int j = 0; j < cnt; ++j) {
    const R *aj = a + b * a_bs + (long long)j * M;
    const S *c1j = c1 + b * c1_bs + (long long)j * M;
    const S *c2j = c2 ? c2 + b * c2_bs + (long long)j * M : nullptr;
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < M;
         r += (long long)nblk * blockDim.x) {
      const double x = (double)aj[r];
      v1 += x * (double)c1j[r];
      if (c2j) v2 += x * (double)c2j[r];
    }
  }
  v1 = block_sum(v1, sh);
  if (threadIdx.x == 0) acc1[b * nblk + blockIdx.x] += v1;
  if (c2) {
    v2 = block_sum(v2, sh);
    if (threadIdx.x == 0) acc2[b * nblk + blockIdx.x] += v2;
  }
}

// out[b] = sum_k partial[b*nblk + k]
__global__ void k_sum_slots(const double *__restrict__ partial, int nblk, double *__restrict__ out) {
  __shared__ double sh[32];
  const int b = blockIdx.x;
  double v = 0.0;
  for (int k = threadIdx.x; k < nblk; k += blockDim.x) v += partial[(long long)b * nblk + k];
  v = block_sum(v, sh);
  if (threadIdx.x == 0) out[b] = v;
}

// adjoint seed at one contour point: out = ffl (cA phibarA + cB phibarB) * v
// (v == null: 1), and the point's contour-weight terms of phi: S += c q q+
template <typename R>
__global__ void k_seed(R *__restrict__ out, const R *__restrict__ v, long long v_bs,
                       const double *__restrict__ pbA, const double *__restrict__ pbB, double cA,
                       double cB, const double *__restrict__ ffl, const R *__restrict__ q,
                       long long q_bs, const R *__restrict__ qc, long long qc_bs,
                       double *__restrict__ SA, double *__restrict__ SB, long long M) {
  const long long b = blockIdx.y;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M;
       i += (long long)gridDim.x * blockDim.x) {
    const long long o = b * M + i;
    const double vv = v ? (double)v[b * v_bs + i] : 1.0;
    out[o] = (R)(ffl[b] * (cA * pbA[o] + cB * pbB[o]) * vv);
    if (SA) {
      const double qq = (double)q[b * q_bs + i] * (qc ? (double)qc[b * qc_bs + i] : 1.0);
      SA[o] += cA * qq;
      SB[o] += cB * qq;
    }
  }
}

// One step of the reverse sweep over the q chain, s -> s-1:
//   wbar += -ds/2 (lam(s) q(s) + (A lam(s)) q(s-1))     (field of step s)
//   G    += q+(s) q(s) + q+(s-1) q(s-1)                (Q part, scaled later)
//   S    += c(s-1) q(s-1) q+(s-1)                        (phi)
//   lam(s-1) = A lam(s) + ffl (cA phibarA + cB phibarB)(s-1) q+(s-1)
template <typename R>
__global__ void k_adj_q(const R *__restrict__ p, const R *__restrict__ lam,
                        const R *__restrict__ qs, const R *__restrict__ qsm1, long long seg_bs,
                        const R *__restrict__ qcs, const R *__restrict__ qcsm1,
                        const double *__restrict__ pbA, const double *__restrict__ pbB,
                        double cA, double cB, const double *__restrict__ ffl, double hds,
                        double *__restrict__ wbar, double *__restrict__ G,
                        double *__restrict__ SA, double *__restrict__ SB, R *__restrict__ lam_out,
                        long long M) {
  const long long b = blockIdx.y;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M;
       i += (long long)gridDim.x * blockDim.x) {
    const long long o = b * M + i, so = b * seg_bs + i;
    const double l = (double)lam[o], pp = (double)p[o], q1 = (double)qs[so],
                 q0 = (double)qsm1[so];
    const double c1 = (double)qcs[o], c0 = (double)qcsm1[o];
    wbar[o] -= hds * (l * q1 + pp * q0);
    G[o] += c1 * q1 + c0 * q0;
    const double qq = q0 * c0;
    SA[o] += cA * qq;
    SB[o] += cB * qq;
    lam_out[o] = (R)(pp + ffl[b] * (cA * pbA[o] + cB * pbB[o]) * c0);
  }
}

// One step of the forward sweep over the q+ chain, s-1 -> s:
//   wbar += -ds/2 (mu(s-1) q+(s-1) + (A mu(s-1)) q+(s))
//   mu(s) = A mu(s-1) + ffl (cA phibarA + cB phibarB)(s) q(s)
template <typename R>
__global__ void k_adj_qc(const R *__restrict__ p, const R *__restrict__ mu,
                         const R *__restrict__ qcsm1, const R *__restrict__ qcs, long long seg_bs,
                         const R *__restrict__ qs, const double *__restrict__ pbA,
                         const double *__restrict__ pbB, double cA, double cB,
                         const double *__restrict__ ffl, double hds, double *__restrict__ wbar,
                         R *__restrict__ mu_out, long long M) {
  const long long b = blockIdx.y;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M;
       i += (long long)gridDim.x * blockDim.x) {
    const long long o = b * M + i, so = b * seg_bs + i;
    const double m = (double)mu[o], pp = (double)p[o];
    wbar[o] -= hds * (m * (double)qcsm1[so] + pp * (double)qcs[so]);
    mu_out[o] = (R)(pp + ffl[b] * (cA * pbA[o] + cB * pbB[o]) * (double)qs[o]);
  }
}

// wbar += coef[b] * G
__global__ void k_axpy_inst(double *__restrict__ wbar, const double *__restrict__ G,
                            const double *__restrict__ coef, long long M) {
  const long long b = blockIdx.y;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M;
       i += (long long)gridDim.x * blockDim.x)
    wbar[b * M + i] += coef[b] * G[b * M + i];
}


}  // namespace

// Work buffers of the adjoint and the stress (working precision R unless
// noted), allocated on first use and kept for later calls.
struct AdjointState {
  size_t bytes = 0;
  void *mem = nullptr;          // one allocation, carved below
  int K = 0, nck1 = 0, nck2 = 0;
  std::vector<int> pos1, pos2;  // checkpoint positions: q at s = pos1[j], q+ at s = N - pos2[j]
  void *ck1 = nullptr, *ck2 = nullptr, *seg = nullptr;
  void *v[12] = {};             // [B][M] vectors
  double *d[10] = {};           // [B][M] FP64 accumulators and seeds
  double *acc = nullptr;        // [kinds][B][nblk]
  double *small = nullptr;      // [8][B]
  // stress chunk buffers
  size_t sbytes = 0, sacc_off = 0;
  void *smem = nullptr;          // chunk x 3 slices, then reduction slots
  int chunk = 0;
};

void scft_internal_adjoint_free(scft_ctx *ctx) {
  if (!ctx->adj) return;
  cudaFree(ctx->adj->mem);
  cudaFree(ctx->adj->smem);
  delete ctx->adj;
  ctx->adj = nullptr;
}

namespace {

constexpr int kAccKinds = 16;
enum AccKind { ACC_L1 = 0, ACC_Q = 3, ACC_L2 = 6, ACC_U1 = 9, ACC_UQ = 10, ACC_U2 = 11,
               ACC_FFL = 12 };

int field_of_step(const scft_ctx *ctx, int s) { return s <= ctx->NsA ? 0 : 1; }

// contour weights of point s in the A and B blocks (those of the forward
// contour sums: trapezoid, or Simpson with SCFT_FLAG_SIMPSON)
void weights(const scft_ctx *ctx, int s, double *cA, double *cB) {
  const bool simpson = (ctx->p.flags & SCFT_FLAG_SIMPSON) != 0;
  *cA = s <= ctx->NsA ? scft::contour_weight(s, ctx->NsA, simpson) : 0.0;
  *cB = s >= ctx->NsA ? scft::contour_weight(s - ctx->NsA, ctx->dNsB, simpson) : 0.0;
}

int ensure_adjoint(scft_ctx *ctx, int K) {
  const int N = ctx->NsA + ctx->dNsB;
  const long long M = ctx->M, B = ctx->batch;
  const size_t rb = ctx->rbytes;
  if (!ctx->adj) ctx->adj = new AdjointState();
  AdjointState &A = *ctx->adj;
  if (A.mem && A.K == K) return SCFT_OK;
  cudaFree(A.mem);
  A.mem = nullptr;
  A.K = K;
  A.pos1.clear();
  for (int s = 0; s < N; s += K) A.pos1.push_back(s);
  A.pos1.push_back(N);
  A.pos2 = A.pos1;      // q+ checkpoints at distance t from the chain end
  A.nck1 = A.nck2 = (int)A.pos1.size();
  const size_t slice = (size_t)M * B * rb;
  const size_t dslice = (size_t)M * B * 8;
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  size_t need = up(slice * A.nck1) + up(slice * A.nck2) + up((size_t)(K + 1) * slice) +
                12 * up(slice) + 10 * up(dslice) + up(8 * (size_t)kAccKinds * B * ctx->nblk) +
                up(8 * (8 + (size_t)kAccKinds) * B);
  CK(cudaMalloc(&A.mem, need));
  A.bytes = need;
  unsigned char *m = static_cast<unsigned char *>(A.mem);
  size_t off = 0;
  auto take = [&](size_t n) { void *p = m + off; off += up(n); return p; };
  A.ck1 = take(slice * A.nck1);
  A.ck2 = take(slice * A.nck2);
  A.seg = take((size_t)(K + 1) * slice);
  for (int i = 0; i < 12; ++i) A.v[i] = take(slice);
  for (int i = 0; i < 10; ++i) A.d[i] = static_cast<double *>(take(dslice));
  A.acc = static_cast<double *>(take(8 * (size_t)kAccKinds * B * ctx->nblk));
  A.small = static_cast<double *>(take(8 * (8 + (size_t)kAccKinds) * B));
  return SCFT_OK;
}

template <typename R>
int adjoint_impl(scft_ctx *ctx, const double *h_pbA, const double *h_pbB, const double *h_Qbar,
                 double *h_wabar, double *h_wbbar, double *h_Lbar) {
  AdjointState &A = *ctx->adj;
  const long long M = ctx->M;
  const int B = ctx->batch, N = ctx->NsA + ctx->dNsB, nblk = ctx->nblk, K = A.K;
  const double ds = ctx->p.ds0, hds = ds / 2;
  cudaStream_t st = ctx->st;
  const bool want_L = h_Lbar != nullptr;
  const int np = (int)ctx->passes.size();
  bool has_unit = false;
  for (int a = 0; a < 3; ++a) has_unit |= ctx->unit_c[a] != 0.0;

  R *ck1 = static_cast<R *>(A.ck1), *ck2 = static_cast<R *>(A.ck2);
  R *seg = static_cast<R *>(A.seg);
  R *W[2] = {static_cast<R *>(A.v[0]), static_cast<R *>(A.v[1])};
  R *va = static_cast<R *>(A.v[2]), *vb = static_cast<R *>(A.v[3]);    // marching pair
  R *x = static_cast<R *>(A.v[4]), *y = static_cast<R *>(A.v[5]);      // on-the-fly chain
  R *l0 = static_cast<R *>(A.v[6]), *l1 = static_cast<R *>(A.v[7]);    // adjoint pair
  R *p = static_cast<R *>(A.v[8]), *t = static_cast<R *>(A.v[9]);
  R *s0 = static_cast<R *>(A.v[10]), *s1 = static_cast<R *>(A.v[11]);
  double *wa_avg = A.d[0], *wbar[2] = {A.d[1], A.d[2]}, *G[2] = {A.d[3], A.d[4]};
  double *SA = A.d[5], *SB = A.d[6], *pbA = A.d[7], *pbB = A.d[8];
  double *acc = A.acc;
  double *Q = A.small, *ffl = A.small + B, *sum = A.small + 2 * B, *coef = A.small + 3 * B;
  double *sums = A.small + 8 * B;   // [kinds][B]
  const long long ckbs1 = (long long)A.nck1 * M, ckbs2 = (long long)A.nck2 * M;
  const long long segbs = (long long)(K + 1) * M;
  const size_t dbytes = sizeof(double) * M * B;
  auto accp = [&](int kind) { return acc + (size_t)kind * B * nblk; };

  // ---- inputs: getConc's mean-free wA (cuda_scft.cu:71), Boltzmann factors, seeds
  CKL(scft::launch_copy_slice<double>(wa_avg, M, ctx->wa, M, M, B, st));
  CKL(scft::launch_partial_sum<double>(wa_avg, M, M, B, ctx->partial, nblk, st));
  CKL(scft::launch_finalize_sum(ctx->partial, nblk, B, 1.0, sum, st));
  CKL(scft::launch_minus_average(wa_avg, sum, M, B, st));
  CKL(scft::launch_boltzmann<R>(wa_avg, W[0], M * B, hds, st));
  CKL(scft::launch_boltzmann<R>(ctx->wb, W[1], M * B, hds, st));
  if (h_pbA) CK(cudaMemcpyAsync(pbA, h_pbA, dbytes, cudaMemcpyHostToDevice, st));
  else CK(cudaMemsetAsync(pbA, 0, dbytes, st));
  if (h_pbB) CK(cudaMemcpyAsync(pbB, h_pbB, dbytes, cudaMemcpyHostToDevice, st));
  else CK(cudaMemsetAsync(pbB, 0, dbytes, st));
  for (double *z : {wbar[0], wbar[1], G[0], G[1], SA, SB}) CK(cudaMemsetAsync(z, 0, dbytes, st));
  CK(cudaMemsetAsync(acc, 0, sizeof(double) * kAccKinds * B * nblk, st));

  auto step = [&](const R *in, long long in_bs, R *out, long long out_bs, int f) {
    return scft_internal_filter(ctx, in, in_bs, out, out_bs, W[f], W[f], M, B, -1, s0, s1, st);
  };
  const dim3 eg(grid_for(M), B);

  // ---- forward: checkpoints of both chains every K steps
  CKL(scft::launch_fill<R>(ck1, M, R(1), ckbs1, B, st));
  CKL(scft::launch_fill<R>(ck2, M, R(1), ckbs2, B, st));
  for (int chain = 0; chain < 2; ++chain) {
    R *ck = chain == 0 ? ck1 : ck2;
    const long long ckbs = chain == 0 ? ckbs1 : ckbs2;
    const std::vector<int> &pos = chain == 0 ? A.pos1 : A.pos2;
    const R *cur = ck;
    long long cur_bs = ckbs;
    size_t j = 1;
    for (int u = 1; u <= N; ++u) {
      const int s = chain == 0 ? u : N - u + 1;   // step applied: q(u-1)->q(u) / q+(s)->q+(s-1)
      R *dst;
      long long dst_bs;
      if (j < pos.size() && pos[j] == u) {
        dst = ck + (long long)j * M;
        dst_bs = ckbs;
        ++j;
      } else {
        dst = (cur == va) ? vb : va;
        dst_bs = M;
      }
      RC(step(cur, cur_bs, dst, dst_bs, field_of_step(ctx, s)));
      cur = dst;
      cur_bs = dst_bs;
    }
  }
  // Q = <q(N)>, ffl = ds/Q (cal_ql and getConc's host lines, cuda_scft.cu:118-125)
  const R *qN = ck1 + (long long)(A.nck1 - 1) * M;
  CKL(scft::launch_partial_sum<R>(qN, ckbs1, M, B, ctx->partial, nblk, st));
  CKL(scft::launch_finalize_sum(ctx->partial, nblk, B, 1.0, sum, st));
  CKL(scft::launch_q_ffl(sum, M, ds, B, Q, ffl, st));

  auto dot = [&](const R *a, long long a_bs, const R *c1, long long c1_bs, const R *c2,
                 long long c2_bs, double *acc1, double *acc2) {
    k_dot_acc<R, R><<<dim3(nblk, B), kT, 0, st>>>(a, a_bs, c1, c1_bs, c2, c2_bs, M, 1, acc1,
                                                   acc2);
    ++ctx->launches;
    return cudaGetLastError();
  };

  // ---- reverse sweep of the q chain (s = N .. 1), q+ marched alongside
  {
    double cA, cB;
    weights(ctx, N, &cA, &cB);
    k_seed<R><<<eg, kT, 0, st>>>(l0, nullptr, 0, pbA, pbB, cA, cB, ffl, qN, ckbs1, nullptr, 0,
                                 SA, SB, M);
    ++ctx->launches;
    CK(cudaGetLastError());
    CKL(scft::launch_fill<R>(x, M * B, R(1), 0, 1, st));
    R *lam = l0, *lam_n = l1, *qc = x, *qc_n = y;
    for (int j = A.nck1 - 2; j >= 0; --j) {
      const int s_lo = A.pos1[j], len = A.pos1[j + 1] - s_lo;
      CKL(scft::launch_copy_slice<R>(seg, segbs, ck1 + (long long)j * M, ckbs1, M, B, st));
      for (int k = 1; k <= len; ++k)
        RC(step(seg + (long long)(k - 1) * M, segbs, seg + (long long)k * M, segbs,
                field_of_step(ctx, s_lo + k)));
      for (int k = len; k >= 1; --k) {
        const int s = s_lo + k, f = field_of_step(ctx, s);
        const R *q1 = seg + (long long)k * M, *q0 = seg + (long long)(k - 1) * M;
        RC(step(qc, M, qc_n, M, f));          // q+(s-1)
        RC(step(lam, M, p, M, f));            // A lam(s)
        if (want_L) {
          for (int pi = 0; pi < np; ++pi) {
            RC(scft_internal_filter(ctx, q0, segbs, t, M, W[f], W[f], M, B, pi, s0, s1, st));
            CK(dot(t, M, lam, M, qc, M, accp(ACC_L1 + pi), accp(ACC_Q + pi)));
          }
          if (has_unit) CK(dot(q1, segbs, lam, M, qc, M, accp(ACC_U1), accp(ACC_UQ)));
        }
        double cA, cB;
        weights(ctx, s - 1, &cA, &cB);
        k_adj_q<R><<<eg, kT, 0, st>>>(p, lam, q1, q0, segbs, qc, qc_n, pbA, pbB, cA, cB, ffl,
                                      hds, wbar[f], G[f], SA, SB, lam_n, M);
        ++ctx->launches;
        CK(cudaGetLastError());
        std::swap(lam, lam_n);
        std::swap(qc, qc_n);
      }
    }
  }
  // ---- forward sweep of the q+ chain (s = 1 .. N), q marched alongside
  {
    double cA, cB;
    weights(ctx, 0, &cA, &cB);
    k_seed<R><<<eg, kT, 0, st>>>(l0, nullptr, 0, pbA, pbB, cA, cB, ffl, nullptr, 0, nullptr, 0,
                                 nullptr, nullptr, M);
    ++ctx->launches;
    CK(cudaGetLastError());
    CKL(scft::launch_fill<R>(x, M * B, R(1), 0, 1, st));
    R *mu = l0, *mu_n = l1, *qv = x, *qv_n = y;
    for (int j = A.nck2 - 2; j >= 0; --j) {
      // segment of q+ at distances t in [pos2[j], pos2[j+1]] from the end
      const int t_lo = A.pos2[j], len = A.pos2[j + 1] - t_lo;
      CKL(scft::launch_copy_slice<R>(seg, segbs, ck2 + (long long)j * M, ckbs2, M, B, st));
      for (int k = 1; k <= len; ++k)
        RC(step(seg + (long long)(k - 1) * M, segbs, seg + (long long)k * M, segbs,
                field_of_step(ctx, N - (t_lo + k) + 1)));
      for (int k = len; k >= 1; --k) {
        const int s = N - (t_lo + k) + 1, f = field_of_step(ctx, s);
        const R *qc0 = seg + (long long)k * M;         // q+(s-1)
        const R *qc1 = seg + (long long)(k - 1) * M;   // q+(s)
        RC(step(qv, M, qv_n, M, f));          // q(s)
        RC(step(mu, M, p, M, f));             // A mu(s-1)
        if (want_L) {
          for (int pi = 0; pi < np; ++pi) {
            RC(scft_internal_filter(ctx, qc1, segbs, t, M, W[f], W[f], M, B, pi, s0, s1, st));
            CK(dot(t, M, mu, M, nullptr, 0, accp(ACC_L2 + pi), nullptr));
          }
          if (has_unit) CK(dot(qc0, segbs, mu, M, nullptr, 0, accp(ACC_U2), nullptr));
        }
        double cA, cB;
        weights(ctx, s, &cA, &cB);
        k_adj_qc<R><<<eg, kT, 0, st>>>(p, mu, qc0, qc1, segbs, qv_n, pbA, pbB, cA, cB, ffl, hds,
                                       wbar[f], mu_n, M);
        ++ctx->launches;
        CK(cudaGetLastError());
        std::swap(mu, mu_n);
        std::swap(qv, qv_n);
      }
    }
  }
  // ---- the Q part: Qbar_tot = Qbar - fflbar ds / Q^2, fflbar = <phibar, S>
  k_dot_acc<double, double><<<dim3(nblk, B), kT, 0, st>>>(pbA, M, SA, M, nullptr, 0, M, 1,
                                                          accp(ACC_FFL), nullptr);
  k_dot_acc<double, double><<<dim3(nblk, B), kT, 0, st>>>(pbB, M, SB, M, nullptr, 0, M, 1,
                                                          accp(ACC_FFL), nullptr);
  ctx->launches += 2;
  CK(cudaGetLastError());
  std::vector<double> sums_h((size_t)kAccKinds * B), hQ(B);
  k_sum_slots<<<kAccKinds * B, kT, 0, st>>>(acc, nblk, sums);
  ++ctx->launches;
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(sums_h.data(), sums, 8 * (size_t)kAccKinds * B, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(hQ.data(), Q, 8 * B, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  std::vector<double> qtot(B), cf(2 * B);
  for (int b = 0; b < B; ++b) {
    const double fflbar = sums_h[(size_t)ACC_FFL * B + b];
    qtot[b] = (h_Qbar ? h_Qbar[b] : 0.0) - fflbar * ds / (hQ[b] * hQ[b]);
    cf[b] = -hds * qtot[b] / (double)M;
  }
  CK(cudaMemcpyAsync(coef, cf.data(), 8 * B, cudaMemcpyHostToDevice, st));
  for (int f = 0; f < 2; ++f) {
    k_axpy_inst<<<eg, kT, 0, st>>>(wbar[f], G[f], coef, M);
    ++ctx->launches;
    CK(cudaGetLastError());
  }
  // getConc's mean subtraction of wA: its adjoint removes the mean of wAbar
  CKL(scft::launch_partial_sum<double>(wbar[0], M, M, B, ctx->partial, nblk, st));
  CKL(scft::launch_finalize_sum(ctx->partial, nblk, B, 1.0, sum, st));
  CKL(scft::launch_minus_average(wbar[0], sum, M, B, st));
  if (h_wabar) CK(cudaMemcpyAsync(h_wabar, wbar[0], dbytes, cudaMemcpyDeviceToHost, st));
  if (h_wbbar) CK(cudaMemcpyAsync(h_wbbar, wbar[1], dbytes, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (want_L) {
    for (int b = 0; b < B; ++b) {
      for (int a = 0; a < 3; ++a) h_Lbar[3 * b + a] = 0.0;
      auto S = [&](int kind) { return sums_h[(size_t)kind * B + b]; };
      for (int pi = 0; pi < np; ++pi)
        h_Lbar[3 * b + ctx->pass_axis[pi]] =
            S(ACC_L1 + pi) + S(ACC_L2 + pi) + qtot[b] / (double)M * S(ACC_Q + pi);
      for (int a = 0; a < 3; ++a)
        if (ctx->unit_c[a] != 0.0)
          h_Lbar[3 * b + a] =
              ctx->unit_c[a] * (S(ACC_U1) + S(ACC_U2) + qtot[b] / (double)M * S(ACC_UQ));
    }
  }
  return SCFT_OK;
}

// Box stress from the propagators stored by the last getConc: for every
// contour step s (all independent, so batched `chunk` steps per launch),
// t = W (dK/dL_a) W q(s-1), contracted with q+(s) in FP64.
template <typename R>
int stress_impl(scft_ctx *ctx, double *h_out) {
  AdjointState &A = *ctx->adj;
  const long long M = ctx->M;
  const int B = ctx->batch, nblk = ctx->nblk, np = (int)ctx->passes.size();
  cudaStream_t st = ctx->st;
  const int chunk = A.chunk;
  R *tb = static_cast<R *>(A.smem);
  R *s0 = tb + (long long)chunk * M, *s1 = s0 + (long long)chunk * M;
  // [4 kinds][B][nblk]: passes 0..2 and the unit term, then [4][B] sums
  double *acc = reinterpret_cast<double *>(static_cast<unsigned char *>(A.smem) + A.sacc_off);
  double *sums = acc + (size_t)4 * B * nblk;
  CK(cudaMemsetAsync(acc, 0, sizeof(double) * 4 * B * nblk, st));
  struct Block { int q, qc, f, ns; };
  const Block blocks[2] = {{SCFT_Q_A, SCFT_Q_CA, 0, ctx->NsA}, {SCFT_Q_B, SCFT_Q_CB, 1, ctx->dNsB}};
  bool has_unit = false;
  for (int a = 0; a < 3; ++a) has_unit |= ctx->unit_c[a] != 0.0;
  for (const Block &bl : blocks) {
    const R *q = static_cast<const R *>(ctx->q[bl.q]);
    const R *qc = static_cast<const R *>(ctx->q[bl.qc]);
    const long long qbs = (long long)(bl.ns + 1) * M;
    const R *Wf = static_cast<const R *>(ctx->W[bl.f]);
    for (int b = 0; b < B; ++b)
      for (int s1st = 1; s1st <= bl.ns; s1st += chunk) {
        const int cnt = std::min(chunk, bl.ns - s1st + 1);
        const R *qin = q + b * qbs + (long long)(s1st - 1) * M;    // q(s-1)
        const R *qcs = qc + b * qbs + (long long)s1st * M;         // q+(s)
        for (int pi = 0; pi < np; ++pi) {
          RC(scft_internal_filter(ctx, qin, M, tb, M, Wf + b * M, Wf + b * M, 0, cnt, pi, s0, s1,
                                  st));
          k_dot_acc<R, R><<<dim3(nblk, 1), kT, 0, st>>>(tb, 0, qcs, 0, nullptr, 0, M, cnt,
                                                        acc + ((size_t)pi * B + b) * nblk,
                                                        nullptr);
          ++ctx->launches;
          CK(cudaGetLastError());
        }
        if (has_unit) {   // W K W q(s-1) = q(s)
          k_dot_acc<R, R><<<dim3(nblk, 1), kT, 0, st>>>(qin + M, 0, qcs, 0, nullptr, 0, M, cnt,
                                                        acc + ((size_t)3 * B + b) * nblk,
                                                        nullptr);
          ++ctx->launches;
          CK(cudaGetLastError());
        }
      }
  }
  std::vector<double> s_h(4 * (size_t)B), hQ(B);
  k_sum_slots<<<4 * B, kT, 0, st>>>(acc, nblk, sums);
  ++ctx->launches;
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(s_h.data(), sums, 8 * 4 * B, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(hQ.data(), ctx->Q, 8 * B, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  for (int b = 0; b < B; ++b) {
    const double scale = -1.0 / ((double)M * hQ[b]);   // -d ln Q / dL
    for (int a = 0; a < 3; ++a) h_out[3 * b + a] = 0.0;
    for (int pi = 0; pi < np; ++pi)
      h_out[3 * b + ctx->pass_axis[pi]] = scale * s_h[(size_t)pi * B + b];
    for (int a = 0; a < 3; ++a)
      if (ctx->unit_c[a] != 0.0) h_out[3 * b + a] = scale * ctx->unit_c[a] * s_h[(size_t)3 * B + b];
  }
  return SCFT_OK;
}

}  // namespace

extern "C" {

int scft_adjoint(scft_ctx *ctx, const double *pha_bar, const double *phb_bar,
                 const double *Q_bar, double *wa_bar, double *wb_bar, double *L_bar,
                 int checkpoint_every) {
  if (!ctx) return SCFT_ERR_INVALID_ARG;
  const int N = ctx->NsA + ctx->dNsB;
  if (N < 1) return scft_fail(ctx, SCFT_ERR_UNSUPPORTED, "adjoint needs at least one step");
  if (checkpoint_every < 0) return scft_fail(ctx, SCFT_ERR_INVALID_ARG, "bad checkpoint interval");
  NvtxRange range("scft adjoint");
  int K = checkpoint_every ? checkpoint_every : (int)ceil(sqrt((double)N));
  if (K > N) K = N;
  CK(cudaSetDevice(ctx->p.device));
  RC(ensure_adjoint(ctx, K));
  return with_real(ctx, [&](auto r) {
    return adjoint_impl<decltype(r)>(ctx, pha_bar, phb_bar, Q_bar, wa_bar, wb_bar, L_bar);
  });
}

int scft_adjoint_checkpoints(scft_ctx *ctx, int checkpoint_every, int *slices,
                             long long *bytes) {
  if (!ctx || !slices) return SCFT_ERR_INVALID_ARG;
  const int N = ctx->NsA + ctx->dNsB;
  int K = checkpoint_every > 0 ? checkpoint_every : (int)ceil(sqrt((double)(N > 0 ? N : 1)));
  if (K > N) K = N > 0 ? N : 1;
  const int nck = (N + K - 1) / K + 1;
  *slices = 2 * nck + K + 1;   // both chains' checkpoints + one recompute segment
  if (bytes) *bytes = (long long)(*slices) * ctx->M * ctx->batch * ctx->rbytes;
  return SCFT_OK;
}

int scft_stress(scft_ctx *ctx, double *dF_dL) {
  if (!ctx || !dF_dL) return SCFT_ERR_INVALID_ARG;
  if (!ctx->have_conc)
    return scft_fail(ctx, SCFT_ERR_INVALID_ARG,
                     "no getConc at the current box: call scft_get_conc first");
  CK(cudaSetDevice(ctx->p.device));
  NvtxRange range("scft stress");
  if (!ctx->adj) ctx->adj = new AdjointState();
  AdjointState &A = *ctx->adj;
  if (!A.smem) {
    // up to 64 contour steps per launch, the three chunk buffers <= 768 MB
    const long long per = ctx->M * ctx->rbytes;
    int chunk = (int)std::min<long long>(64, std::max<long long>(1, (256LL << 20) / per));
    chunk = std::min(chunk, std::max(ctx->NsA, ctx->dNsB));
    chunk = std::max(chunk, 1);
    A.chunk = chunk;
    A.sacc_off = ((size_t)3 * chunk * per + 255) & ~(size_t)255;
    A.sbytes = A.sacc_off + 8 * ((size_t)4 * ctx->batch * ctx->nblk + 4 * ctx->batch);
    CK(cudaMalloc(&A.smem, A.sbytes));
  }
  return with_real(ctx, [&](auto r) { return stress_impl<decltype(r)>(ctx, dF_dL); });
}

int scft_relax_cell(scft_ctx *ctx, int axes_mask, double tol_w, double tol_stress,
                    int max_outer, int max_inner, double step0, int *outer_iters,
                    double *dF_dL, double *out5) {
  if (!ctx || !(tol_w > 0) || !(tol_stress > 0) || max_outer < 1 || max_inner < 1 ||
      !(step0 > 0) || (axes_mask & ~7) || !axes_mask)
    return SCFT_ERR_INVALID_ARG;
  if (ctx->batch != 1)
    return scft_fail(ctx, SCFT_ERR_UNSUPPORTED, "cell relaxation needs batch == 1 (one box)");
  double L[3] = {ctx->p.lx, ctx->p.ly, ctx->p.lz}, sig[3], fe[5];
  double L_prev[3] = {0, 0, 0}, sig_prev[3] = {0, 0, 0};
  double alpha = step0;
  // Inexact inner solves: far from the stress-free box the fields need not be
  // converged tightly, so each round converges to max(tol_w, stress/10) of
  // the previous round (at most 1e-3); the last round always reaches tol_w.
  double tol = std::max(tol_w, 1e-3);
  int it = 0;
  for (;;) {
    int iters = 0;
    RC(scft_converge(ctx, tol, max_inner, &iters, fe));
    RC(scft_internal_get_conc(ctx));   // propagators of the converged fields
    RC(scft_stress(ctx, sig));
    double smax = 0.0;
    for (int a = 0; a < 3; ++a)
      if (axes_mask >> a & 1) smax = std::max(smax, fabs(sig[a]));
    ++it;
    if (it >= max_outer) break;
    if (smax < tol_stress) {
      if (tol <= tol_w) break;
      tol = tol_w;   // stress-free at a loose tolerance: tighten, same box
      continue;
    }
    tol = std::max(tol_w, std::min(1e-3, 0.1 * smax));
    // Barzilai-Borwein step on F*(L), whose gradient is the stress
    if (it > 1) {
      double ss = 0.0, sy = 0.0;
      for (int a = 0; a < 3; ++a)
        if (axes_mask >> a & 1) {
          const double dl = L[a] - L_prev[a], dg = sig[a] - sig_prev[a];
          ss += dl * dl;
          sy += dl * dg;
        }
      if (sy > 0.0) alpha = ss / sy;
    }
    double Ln[3] = {L[0], L[1], L[2]};
    for (int a = 0; a < 3; ++a) {
      if (!(axes_mask >> a & 1)) continue;
      double d = -alpha * sig[a];
      const double cap = 0.05 * L[a];   // at most 5% per step
      d = std::max(-cap, std::min(cap, d));
      Ln[a] = L[a] + d;
    }
    for (int a = 0; a < 3; ++a) {
      L_prev[a] = L[a];
      sig_prev[a] = sig[a];
      L[a] = Ln[a];
    }
    RC(scft_set_box(ctx, L[0], L[1], L[2]));
  }
  if (outer_iters) *outer_iters = it;
  if (dF_dL) for (int a = 0; a < 3; ++a) dF_dL[a] = sig[a];
  if (out5) for (int k = 0; k < 5; ++k) out5[k] = fe[k];
  return SCFT_OK;
}

}  // extern "C"
