// C ABI of the SCFT hot path (include/scft_capi.h): context set-up, the
// propagator march, getConc, mixing, free energy and the SCF loop.  Host
// code only; kernels live in k_line.cu / k_fields.cu.
#include <math.h>
#include <chrono>
#include <cmath>
#include <stdio.h>
#include <string.h>

#include <string>
#include <type_traits>
#include <vector>

#include "ctx.h"

using scft::AxisPlan;

namespace {

// struct.h:11 -- the reference's value of pi, used for the wave numbers.
constexpr double kPiRef = 3.1415926535;

// per host thread: contexts may be created from several threads at once
thread_local std::string g_create_err = "no error";

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

// Squared wave numbers of one axis, in the reference's order of operations
// (init_cuda.cu:398-418): bins i <= n/2-1 are +i, bins i >= n/2 are i-n.
std::vector<double> k2_axis(int n, double L) {
  std::vector<double> k(n);
  const double d = L / n;
  for (int i = 0; i <= n / 2 - 1; ++i) k[i] = 2 * kPiRef * i * 1.0 / n / d;
  for (int i = n / 2; i < n; ++i) k[i] = 2 * kPiRef * (i - n) * 1.0 / d / n;
  for (int i = 0; i < n; ++i) k[i] *= k[i];
  return k;
}

// Gains of the passes (kxyzdz, init_cuda.cu:394-428, split per axis:
// exp(-ds0 k^2)/n, with the constant factors of length-1 axes folded into the
// first pass) and their box derivatives: d/dL_a of exp(-ds0 k_a^2) is
// exp(-ds0 k_a^2) * 2 ds0 k_a^2 / L_a because k_a is proportional to 1/L_a.
// Rewritten in place when the box changes.
int upload_gains(scft_ctx *ctx) {
  const scft_params &p = ctx->p;
  const int dims[3] = {p.nx, p.ny, p.nz};
  const double lens[3] = {p.lx, p.ly, p.lz};
  const size_t rb = ctx->rbytes;
  double scalar = 1.0;
  for (int a = 0; a < 3; ++a) {
    ctx->unit_c[a] = 0.0;
    if (dims[a] == 1) {
      const double k2 = k2_axis(1, lens[a])[0];
      scalar *= exp(-p.ds0 * k2);
      ctx->unit_c[a] = 2.0 * p.ds0 * k2 / lens[a];
    }
  }
  size_t dbytes = 0;
  for (const AxisPlan &ap : ctx->passes) dbytes += ((size_t)ap.n * rb + 255) & ~(size_t)255;
  if (!ctx->dgain) CK(cudaMalloc(&ctx->dgain, dbytes));
  size_t doff = 0;
  for (size_t pi = 0; pi < ctx->passes.size(); ++pi) {
    const AxisPlan &ap = ctx->passes[pi];
    const int a = ctx->pass_axis[pi];
    const std::vector<double> k2 = k2_axis(ap.n, lens[a]);
    std::vector<double> g(ap.n), dg(ap.n);
    for (int m = 0; m < ap.n; ++m) {
      g[m] = exp(-p.ds0 * k2[m]) / ap.n;
      if (pi == 0) g[m] *= scalar;
      dg[m] = g[m] * 2.0 * p.ds0 * k2[m] / lens[a];
    }
    void *dptr = static_cast<unsigned char *>(ctx->dgain) + doff;
    ctx->dgain_pass[pi] = dptr;
    doff += ((size_t)ap.n * rb + 255) & ~(size_t)255;
    if (rb == 4) {
      std::vector<float> gf(g.begin(), g.end()), dgf(dg.begin(), dg.end());
      CK(cudaMemcpy(const_cast<void *>(ap.gain), gf.data(), 4 * ap.n, cudaMemcpyHostToDevice));
      CK(cudaMemcpy(dptr, dgf.data(), 4 * ap.n, cudaMemcpyHostToDevice));
    } else if (ctx->rkind == kRealDF) {
      std::vector<scft::dfloat> gd(g.begin(), g.end()), dgd(dg.begin(), dg.end());
      CK(cudaMemcpy(const_cast<void *>(ap.gain), gd.data(), 8 * ap.n, cudaMemcpyHostToDevice));
      CK(cudaMemcpy(dptr, dgd.data(), 8 * ap.n, cudaMemcpyHostToDevice));
    } else {
      CK(cudaMemcpy(const_cast<void *>(ap.gain), g.data(), 8 * ap.n, cudaMemcpyHostToDevice));
      CK(cudaMemcpy(dptr, dg.data(), 8 * ap.n, cudaMemcpyHostToDevice));
    }
  }
  return SCFT_OK;
}

bool radix_plan(int n, int *fac, int *nfac) {
  int m = n, k = 0;
  while (m % 4 == 0) { fac[k++] = 4; m /= 4; }
  while (m % 2 == 0) { fac[k++] = 2; m /= 2; }
  for (int p = 3; p <= 61 && m > 1; p += 2) {
    while (m % p == 0) {
      if (k >= 24) return false;
      fac[k++] = p;
      m /= p;
    }
  }
  *nfac = k;
  return m == 1;
}

bool axis_ok(int n, bool allow_one) {
  if (n == 1) return allow_one;
  if (n < 2 || (n & 1)) return false;
  if (n > 4096) return false;
  int fac[24], nf;
  return radix_plan(n, fac, &nf);
}

// One pass over a set of propagators: a single launch of the register
// kernel, or one generic launch per set member.
template <typename R>
int launch_set(scft_ctx *ctx, const AxisPlan &ap, const scft::PassSet<R> &ps, cudaStream_t st) {
  if (ap.use_fast) {
    CKL(scft::launch_fast_line(ap, ps, st));
    return SCFT_OK;
  }
  if constexpr (std::is_same<R, scft::dfloat>::value) {
    // scft_create admits double-float contexts only when every pass is fast
    return scft_fail(ctx, SCFT_ERR_UNSUPPORTED, "double-float pass without a register kernel");
  } else {
  for (int k = 0; k < ps.nset; ++k)
    CKL(scft::launch_line_filter<R>(ap, ps.in[k], ps.in_bs[k], ps.out[k], ps.out_bs[k],
                                    ps.pre[k], ps.post[k], ps.w_bs, ps.batch, st));
  return SCFT_OK;
  }
}

// A march segment: propagator qi over ns steps in field wf, direction sign,
// starting from slice is of propagator iq (iq < 0: qInt = 1, qInt_init,
// cuda_aid.cu:197-208; iq == 4: the qInt buffer).
struct Seg {
  int qi, wf, iq, is, ns, sign;
};

// initilize_q / initilize_q_inverse (cuda_scft.cu:463,513) of a segment.
template <typename R>
int seg_boundary(scft_ctx *ctx, const Seg &s, cudaStream_t st) {
  const long long M = ctx->M;
  const int B = ctx->batch;
  R *q = static_cast<R *>(ctx->q[s.qi]);
  const long long qbs = (long long)(ctx->q_ns[s.qi] + 1) * M;
  R *dst = q + (long long)(s.sign > 0 ? 0 : s.ns) * M;
  if (s.iq < 0) {
    CKL(scft::launch_fill<R>(dst, M, R(1), qbs, B, st));
  } else {
    const R *src = s.iq == 4 ? static_cast<const R *>(ctx->qint)
                             : static_cast<const R *>(ctx->q[s.iq]) + (long long)s.is * M;
    const long long sbs = s.iq == 4 ? M : (long long)(ctx->q_ns[s.iq] + 1) * M;
    CKL(scft::launch_copy_slice<R>(dst, qbs, src, sbs, M, B, st));
  }
  return SCFT_OK;
}

// Runs up to kMaxSet chains of march segments in lockstep: contour step t of
// every chain is one set of pass launches (sovDifFft's per-step
// initilize_in_go -> D2Z -> sufaceField_go -> Z2D -> in_to_g_go,
// cuda_scft.cu:467-491, as one line-filter pass per axis).  Chains are
// independent, so the interleaving does not change any result.
template <typename R>
int run_chains(scft_ctx *ctx, const Seg *const *chains, const int *nseg, int nchain,
               cudaStream_t st, int chain_base) {
  const long long M = ctx->M;
  int total[scft::kMaxSet] = {0, 0};
  int maxT = 0;
  for (int c = 0; c < nchain; ++c) {
    for (int k = 0; k < nseg[c]; ++k) total[c] += chains[c][k].ns;
    if (total[c] > maxT) maxT = total[c];
    int rc = seg_boundary<R>(ctx, chains[c][0], st);
    if (rc) return rc;
  }
  // stages per step: the x and y passes fused into one plane kernel when
  // possible (FP32), then the remaining passes
  const bool xy = sizeof(R) == 4 && ctx->fuse_xy;
  const int np = (int)ctx->passes.size() - (xy ? 1 : 0);
  for (int t = 1; t <= maxT; ++t) {
    scft::PassSet<R> ps[3];
    int nact = 0;
    R *q_dst[scft::kMaxSet];
    const R *q_src[scft::kMaxSet], *W[scft::kMaxSet];
    long long qbs[scft::kMaxSet];
    int cidx[scft::kMaxSet];
    for (int c = 0; c < nchain; ++c) {
      if (t > total[c]) continue;
      int k = 0, it = t;
      while (it > chains[c][k].ns) it -= chains[c][k++].ns;
      const Seg &s = chains[c][k];
      if (it == 1 && k > 0) {
        int rc = seg_boundary<R>(ctx, s, st);
        if (rc) return rc;
      }
      const int dst = s.sign > 0 ? it : s.ns - it;
      const int src = s.sign > 0 ? dst - 1 : dst + 1;
      R *q = static_cast<R *>(ctx->q[s.qi]);
      qbs[nact] = (long long)(ctx->q_ns[s.qi] + 1) * M;
      q_dst[nact] = q + (long long)dst * M;
      q_src[nact] = q + (long long)src * M;
      W[nact] = static_cast<const R *>(ctx->W[s.wf]);
      cidx[nact] = c + chain_base;   // selects the chain's intermediates
      ++nact;
    }
    for (int pi = 0; pi < np; ++pi) {
      scft::PassSet<R> &p = ps[pi];
      memset(&p, 0, sizeof(p));
      p.nset = nact;
      p.batch = ctx->batch;
      p.w_bs = M;
      p.err = ctx->use_pipe ? ctx->dev_err : nullptr;
      for (int a = 0; a < nact; ++a) {
        R *tmp0 = static_cast<R *>(ctx->tmp[2 * cidx[a]]);
        R *tmp1 = static_cast<R *>(ctx->tmp[2 * cidx[a] + 1]);
        p.in[a] = pi == 0 ? q_src[a] : ((pi - 1) & 1 ? tmp1 : tmp0);
        p.in_bs[a] = pi == 0 ? qbs[a] : M;
        p.out[a] = pi == np - 1 ? q_dst[a] : (pi & 1 ? tmp1 : tmp0);
        p.out_bs[a] = pi == np - 1 ? qbs[a] : M;
        p.pre[a] = pi == 0 ? W[a] : nullptr;
        p.post[a] = pi == np - 1 ? W[a] : nullptr;
      }
      int rc;
      if constexpr (sizeof(R) == 4) {
        if (xy && pi == 0) {
          CKL(scft::launch_xy(ctx->passes[0], ctx->passes[1], p, st));
          continue;
        }
      }
      rc = launch_set<R>(ctx, ctx->passes[xy ? pi + 1 : pi], p, st);
      if (rc) return rc;
    }
  }
  return SCFT_OK;
}

// One chain with fused step pairs (FP32, x+y plane fusion, fast z pass):
// within a segment, step k runs its passes in the order (x+y, z) when k is
// odd and (z, x+y) when k is even, which the commuting axis filters allow.
// The end of step k and the start of step k+1 are then one kernel
// (k_zz / k_xyxy): one launch per contour step instead of two.
// Without the x+y plane (three passes, all register-resident) the same idea
// gives (x, y, z) for odd and (z, y, x) for even steps: k_zz / k_xx fuse the
// end of one step with the start of the next, two launches per step instead
// of three.
bool fused_possible(const scft_ctx *ctx) {
  if (!ctx->fuse_steps || ctx->passes.size() != 3) return false;
  if (ctx->fuse_xy) return ctx->rbytes == 4 && ctx->passes[2].use_fast != 0;
  return ctx->passes[0].use_fast && ctx->passes[1].use_fast && ctx->passes[2].use_fast;
}

template <typename R>
int run_chain_fused_axes(scft_ctx *ctx, const Seg *segs, int nseg, cudaStream_t st, int cidx) {
  const long long M = ctx->M;
  R *tmp[2] = {static_cast<R *>(ctx->tmp[2 * cidx]), static_cast<R *>(ctx->tmp[2 * cidx + 1])};
  const AxisPlan &apx = ctx->passes[0], &apy = ctx->passes[1], &apz = ctx->passes[2];
  for (int k = 0; k < nseg; ++k) {
    const Seg &sg = segs[k];
    int rc = seg_boundary<R>(ctx, sg, st);
    if (rc) return rc;
    if (sg.ns == 0) continue;
    R *q = static_cast<R *>(ctx->q[sg.qi]);
    const long long qbs = (long long)(ctx->q_ns[sg.qi] + 1) * M;
    const R *W = static_cast<const R *>(ctx->W[sg.wf]);
    auto slice = [&](int it) { return q + (long long)(sg.sign > 0 ? it : sg.ns - it) * M; };
    scft::PassSet<R> ps;
    auto reset = [&](const R *in, long long in_bs, R *out, long long out_bs) {
      memset(&ps, 0, sizeof(ps));
      ps.nset = 1;
      ps.batch = ctx->batch;
      ps.w_bs = M;
      ps.in[0] = in;
      ps.in_bs[0] = in_bs;
      ps.out[0] = out;
      ps.out_bs[0] = out_bs;
    };
    // step 1: x with the pre factor, then y; tmp[0] holds the state between steps
    reset(slice(0), qbs, tmp[1], M);
    ps.pre[0] = W;
    if ((rc = launch_set<R>(ctx, apx, ps, st))) return rc;
    reset(tmp[1], M, tmp[0], M);
    if ((rc = launch_set<R>(ctx, apy, ps, st))) return rc;
    for (int it = 2; it <= sg.ns; ++it) {
      // finish step it-1 (z when it was odd, x when even) and start step it
      reset(tmp[0], M, tmp[1], M);
      ps.qout[0] = slice(it - 1);
      ps.qout_bs[0] = qbs;
      ps.post[0] = W;
      if ((it - 1) & 1) CKL(scft::launch_zz(apz, ps, st));
      else CKL(scft::launch_xx(apx, ps, st));
      reset(tmp[1], M, tmp[0], M);
      if ((rc = launch_set<R>(ctx, apy, ps, st))) return rc;
    }
    reset(tmp[0], M, slice(sg.ns), qbs);
    ps.post[0] = W;
    if ((rc = launch_set<R>(ctx, (sg.ns & 1) ? apz : apx, ps, st))) return rc;
  }
  return SCFT_OK;
}

int run_chain_fused(scft_ctx *ctx, const Seg *segs, int nseg, cudaStream_t st, int cidx) {
  if (!ctx->fuse_xy)
    return with_real(ctx, [&](auto r) {
      return run_chain_fused_axes<decltype(r)>(ctx, segs, nseg, st, cidx);
    });
  const long long M = ctx->M;
  float *tmp[2] = {static_cast<float *>(ctx->tmp[2 * cidx]),
                   static_cast<float *>(ctx->tmp[2 * cidx + 1])};
  const AxisPlan &apx = ctx->passes[0], &apy = ctx->passes[1], &apz = ctx->passes[2];
  for (int k = 0; k < nseg; ++k) {
    const Seg &sg = segs[k];
    int rc = seg_boundary<float>(ctx, sg, st);
    if (rc) return rc;
    if (sg.ns == 0) continue;
    float *q = static_cast<float *>(ctx->q[sg.qi]);
    const long long qbs = (long long)(ctx->q_ns[sg.qi] + 1) * M;
    const float *W = static_cast<const float *>(ctx->W[sg.wf]);
    auto slice = [&](int it) { return q + (long long)(sg.sign > 0 ? it : sg.ns - it) * M; };
    scft::PassSet<float> ps;
    auto reset = [&]() {
      memset(&ps, 0, sizeof(ps));
      ps.nset = 1;
      ps.batch = ctx->batch;
      ps.w_bs = M;
    };
    int cur = 0;
    // step 1 starts with x+y and the pre factor
    reset();
    ps.in[0] = slice(0);
    ps.in_bs[0] = qbs;
    ps.out[0] = tmp[cur];
    ps.out_bs[0] = M;
    ps.pre[0] = W;
    CKL(scft::launch_xy(apx, apy, ps, st));
    for (int it = 2; it <= sg.ns; ++it) {
      // finish step it-1, start step it
      reset();
      ps.in[0] = tmp[cur];
      ps.in_bs[0] = M;
      ps.out[0] = tmp[cur ^ 1];
      ps.out_bs[0] = M;
      ps.qout[0] = slice(it - 1);
      ps.qout_bs[0] = qbs;
      ps.post[0] = W;
      if ((it - 1) & 1) CKL(scft::launch_zz(apz, ps, st));     // step it-1 was (x+y, z)
      else CKL(scft::launch_xyxy(apx, apy, ps, st));            // step it-1 was (z, x+y)
      cur ^= 1;
    }
    // finish the last step with its remaining pass and the post factor
    reset();
    ps.in[0] = tmp[cur];
    ps.in_bs[0] = M;
    ps.out[0] = slice(sg.ns);
    ps.out_bs[0] = qbs;
    ps.post[0] = W;
    if (sg.ns & 1) {
      rc = launch_set<float>(ctx, apz, ps, st);
      if (rc) return rc;
    } else {
      CKL(scft::launch_xy(apx, apy, ps, st));
    }
  }
  return SCFT_OK;
}

int run_chains_any(scft_ctx *ctx, const Seg *const *chains, const int *nseg, int nchain,
                   cudaStream_t st, int chain_base = 0) {
  if (nchain == 1 && fused_possible(ctx))
    return run_chain_fused(ctx, chains[0], nseg[0], st, chain_base);
  return with_real(ctx, [&](auto r) {
    return run_chains<decltype(r)>(ctx, chains, nseg, nchain, st, chain_base);
  });
}

// initilize_wdz (cuda_scft.cu:450) for field f into W[f].
int boltzmann(scft_ctx *ctx, int f, cudaStream_t st) {
  const double *w = f == SCFT_FIELD_WA ? ctx->wa : ctx->wb;
  return with_real(ctx, [&](auto r) {
    using R = decltype(r);
    CKL(scft::launch_boltzmann<R>(w, static_cast<R *>(ctx->W[f]), ctx->M * ctx->batch,
                                  ctx->p.ds0 / 2, st));
    return SCFT_OK;
  });
}

// The march phase of getConc (cuda_scft.cu:77-112) as two lockstep chains:
// qA (from 1) then qB (from qA[NsA]); q+B (from 1) then q+A (from q+B[0]).
// Each march gets exactly the inputs of the reference's sequential order.
int march_phase(scft_ctx *ctx, cudaStream_t st) {
  const Seg c0[2] = {{SCFT_Q_A, SCFT_FIELD_WA, -1, 0, ctx->NsA, 1},
                     {SCFT_Q_B, SCFT_FIELD_WB, SCFT_Q_A, ctx->NsA, ctx->dNsB, 1}};
  const Seg c1[2] = {{SCFT_Q_CB, SCFT_FIELD_WB, -1, 0, ctx->dNsB, -1},
                     {SCFT_Q_CA, SCFT_FIELD_WA, SCFT_Q_CB, 0, ctx->NsA, -1}};
  const Seg *chains[2] = {c0, c1};
  const int nseg[2] = {2, 2};
  if (!ctx->two_streams) return run_chains_any(ctx, chains, nseg, 2, st);
  // the chains on two forked streams: each pass launch of one chain can fill
  // the SMs left idle by the tail of the other chain's launch
  CK(cudaEventRecord(ctx->ev_fork, st));
  CK(cudaStreamWaitEvent(ctx->st2, ctx->ev_fork, 0));
  int rc = run_chains_any(ctx, &chains[0], &nseg[0], 1, st, 0);
  if (!rc) rc = run_chains_any(ctx, &chains[1], &nseg[1], 1, ctx->st2, 1);
  CK(cudaEventRecord(ctx->ev_join, ctx->st2));
  CK(cudaStreamWaitEvent(st, ctx->ev_join, 0));
  return rc;
}

// The march phase through a CUDA graph captured on first use (the pointers
// and step counts of a context never change), so one launch replays the
// ~3*(NsA+dNsB) kernels of the phase.
int march_phase_graph(scft_ctx *ctx) {
  NvtxRange range("scft march phase");
  if (!ctx->use_graph || ctx->capturing) return march_phase(ctx, ctx->st);
  if (!ctx->march_exec) {
    const long long l0 = ctx->launches;
    CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
    int rc = march_phase(ctx, ctx->st);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->st, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess)
      return scft_fail(ctx, SCFT_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&ctx->march_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      ctx->march_exec = nullptr;
      return scft_fail(ctx, SCFT_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    }
    ctx->march_nodes = ctx->launches - l0;
    ctx->launches = l0;
  }
  CK(cudaGraphLaunch(ctx->march_exec, ctx->st));
  ctx->launches += ctx->march_nodes;
  return SCFT_OK;
}

int prof_reserve(scft_ctx *ctx, size_t n_events) {
  while (ctx->prof_events.size() < n_events) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    ctx->prof_events.push_back(e);
  }
  return SCFT_OK;
}

int prof_begin(scft_ctx *ctx) {
  if (!ctx->profiling) return SCFT_OK;
  int rc = prof_reserve(ctx, ctx->prof_used + 2);
  if (rc) return rc;
  CK(cudaEventRecord(ctx->prof_events[ctx->prof_used], ctx->st));
  return SCFT_OK;
}
int prof_end(scft_ctx *ctx, double point_steps) {
  if (!ctx->profiling) return SCFT_OK;
  CK(cudaEventRecord(ctx->prof_events[ctx->prof_used + 1], ctx->st));
  ctx->prof_used += 2;
  ctx->prof_point_steps += point_steps;
  return SCFT_OK;
}

// The public single march (scft_sov_dif_fft): W from the field, init = qInt.
int march(scft_ctx *ctx, int qi, int w_field, int ns, int sign) {
  int rc;
  if ((rc = boltzmann(ctx, w_field, ctx->st))) return rc;
  if ((rc = prof_begin(ctx))) return rc;
  const Seg s[1] = {{qi, w_field, 4, 0, ns, sign}};
  const Seg *chains[1] = {s};
  const int nseg[1] = {1};
  if ((rc = run_chains_any(ctx, chains, nseg, 1, ctx->st))) return rc;
  return prof_end(ctx, (double)ns * ctx->M * ctx->batch);
}

int average(scft_ctx *ctx, double *data) {
  CKL(scft::launch_partial_sum<double>(data, ctx->M, ctx->M, ctx->batch, ctx->partial, ctx->nblk,
                                       ctx->st));
  CKL(scft::launch_finalize_sum(ctx->partial, ctx->nblk, ctx->batch, 1.0, ctx->sum, ctx->st));
  CKL(scft::launch_minus_average(data, ctx->sum, ctx->M, ctx->batch, ctx->st));
  return SCFT_OK;
}

int set_qint(scft_ctx *ctx, int qi, int s) {
  const long long M = ctx->M;
  return with_real(ctx, [&](auto r) {
    using R = decltype(r);
    if (qi < 0) {
      CKL(scft::launch_fill<R>(static_cast<R *>(ctx->qint), M, R(1.0f), M, ctx->batch, ctx->st));
      return SCFT_OK;
    }
    const long long qbs = (long long)(ctx->q_ns[qi] + 1) * M;
    CKL(scft::launch_copy_slice<R>(static_cast<R *>(ctx->qint), M,
                                   static_cast<R *>(ctx->q[qi]) + (long long)s * M, qbs, M,
                                   ctx->batch, ctx->st));
    return SCFT_OK;
  });
}

template <typename R>
int q_and_phi(scft_ctx *ctx) {
  const long long M = ctx->M;
  const int B = ctx->batch;
  // cal_ql on qb[dNsB] (cuda_scft.cu:118), then ql/M and ffl=ds0/Q (:123-126)
  const R *qb = static_cast<const R *>(ctx->q[SCFT_Q_B]);
  const long long qbs = (long long)(ctx->q_ns[SCFT_Q_B] + 1) * M;
  CKL(scft::launch_partial_sum<R>(qb + (long long)ctx->dNsB * M, qbs, M, B, ctx->partial,
                                  ctx->nblk, ctx->st));
  CKL(scft::launch_finalize_sum(ctx->partial, ctx->nblk, B, 1.0, ctx->sum, ctx->st));
  CKL(scft::launch_q_ffl(ctx->sum, M, ctx->p.ds0, B, ctx->Q, ctx->ffl, ctx->st));
  // w_to_phi_go (cuda_scft.cu:130)
  const bool simpson = (ctx->p.flags & SCFT_FLAG_SIMPSON) != 0;
  CKL(scft::launch_contour_phi<R>(static_cast<const R *>(ctx->q[SCFT_Q_A]),
                                  static_cast<const R *>(ctx->q[SCFT_Q_CA]), ctx->NsA, M, B,
                                  ctx->ffl, ctx->pha, simpson, ctx->st));
  CKL(scft::launch_contour_phi<R>(static_cast<const R *>(ctx->q[SCFT_Q_B]),
                                  static_cast<const R *>(ctx->q[SCFT_Q_CB]), ctx->dNsB, M, B,
                                  ctx->ffl, ctx->phb, simpson, ctx->st));
  return SCFT_OK;
}

// getConc (cuda_scft.cu:61-138): average_value(wa), the Boltzmann factors
// (initilize_wdz, :450, once per field instead of once per march), the march
// phase, then Q and the contour sums.
int get_conc(scft_ctx *ctx) {
  NvtxRange range("scft getConc");
  int rc;
  if ((rc = average(ctx, ctx->wa))) return rc;                                 // :71
  if ((rc = boltzmann(ctx, SCFT_FIELD_WA, ctx->st))) return rc;
  if ((rc = boltzmann(ctx, SCFT_FIELD_WB, ctx->st))) return rc;
  if ((rc = prof_begin(ctx))) return rc;
  if ((rc = march_phase_graph(ctx))) return rc;                                // :77-112
  if ((rc = prof_end(ctx, 2.0 * (ctx->NsA + ctx->dNsB) * ctx->M * ctx->batch))) return rc;
  rc = with_real(ctx, [&](auto r) { return q_and_phi<decltype(r)>(ctx); });
  ctx->have_conc = rc == SCFT_OK;
  return rc;
}

// The field update.  Simple mixing is phi_w (cuda_aid.cu:382-416) with its
// residual reduced on the way; Anderson mixing stores (w + lambda d, d) in the
// ring, extends the FP64 Gram matrix by one row, solves the small
// least-squares problem on the device and applies the mixed step.  No host
// round trip.
int mix(scft_ctx *ctx) {
  NvtxRange range("scft field update");
  const long long M = ctx->M;
  const int B = ctx->batch;
  if (ctx->p.mixing == SCFT_MIX_CONSTRAINED || ctx->p.mixing == SCFT_MIX_CONSTRAINED_EX) {
    // the residual of the free update (for convergence reports), then the
    // constrained step
    if (!ctx->target)
      return scft_fail(ctx, SCFT_ERR_INVALID_ARG, "constrained mixing needs a target field");
    CKL(scft::launch_residual(ctx->wa, ctx->wb, ctx->pha, ctx->phb, ctx->p.hAB, ctx->p.wcmp, 0.0,
                              M, B, nullptr, nullptr, 0.0, nullptr, ctx->rpartial, ctx->nblk,
                              ctx->res, ctx->st));
    CKL(scft::launch_phi_w_constrained(ctx->wa, ctx->wb, ctx->pha, ctx->phb, ctx->target,
                                       ctx->p.hAB, ctx->p.constraint_lambda,
                                       ctx->p.mixing == SCFT_MIX_CONSTRAINED_EX, M, B, ctx->st));
    ctx->launches += 3;
    return SCFT_OK;
  }
  if (ctx->p.mixing == SCFT_MIX_SIMPLE) {
    CKL(scft::launch_residual(ctx->wa, ctx->wb, ctx->pha, ctx->phb, ctx->p.hAB, ctx->p.wcmp,
                              ctx->p.wopt, M, B, nullptr, nullptr, 0.0, nullptr, ctx->rpartial,
                              ctx->nblk, ctx->res, ctx->st));
    ctx->launches += 3;   // launch_residual issues four kernels
    return SCFT_OK;
  }
  const int m = ctx->p.anderson_history, m1 = ctx->m1;
  const int c = (int)(ctx->and_count % m1);
  const int hist = (int)(ctx->and_count < m ? ctx->and_count : m);
  CKL(scft::launch_residual(ctx->wa, ctx->wb, ctx->pha, ctx->phb, ctx->p.hAB, ctx->p.wcmp, 0.0,
                            M, B, ctx->hist_u[c], ctx->hist_d[c], ctx->p.anderson_lambda,
                            ctx->wprev, ctx->rpartial, ctx->nblk, ctx->res, ctx->st));
  const void *dj[33], *uj[33];
  int slots[33];
  for (int k = 0; k <= hist; ++k) {
    const int j = ((c - k) % m1 + m1) % m1;
    slots[k] = j;
    dj[k] = ctx->hist_d[j];
    uj[k] = ctx->hist_u[j];
  }
  CKL(scft::launch_gram_row(ctx->hist_d[c], dj, slots, hist + 1, c, m1, M, B, ctx->rpartial,
                            ctx->nblk, ctx->gram, ctx->st));
  CKL(scft::launch_anderson_solve(ctx->gram, ctx->res, c, hist, m1, ctx->p.anderson_start,
                                  ctx->p.anderson_lambda, ctx->p.wopt, B, ctx->and_a,
                                  ctx->and_lam, ctx->st));
  CKL(scft::launch_anderson_update(ctx->wa, ctx->wb, uj, ctx->hist_d[c], slots, hist + 1,
                                   ctx->and_a, ctx->and_lam, m1, M, B, ctx->st));
  ctx->launches += 4;   // residual: 4 kernels, Gram row: 2
  if (ctx->p.flags & SCFT_FLAG_PIN_TRANSLATION) {
    // the update without its rigid-shift component; wprev holds the
    // pre-update fields
    CKL(scft::launch_remove_translation(ctx->wa, ctx->wb, ctx->wprev, ctx->p.nx, ctx->p.ny,
                                        ctx->p.nz, B, ctx->rpartial, ctx->nblk, ctx->shift_alpha,
                                        ctx->st));
    ctx->launches += 2;
  }
  ctx->and_count++;
  return SCFT_OK;
}

int free_energy_dev(scft_ctx *ctx) {
  CKL(scft::launch_free_energy_partials(ctx->wa, ctx->wb, ctx->pha, ctx->phb, ctx->p.hAB, ctx->M,
                                        ctx->batch, ctx->partial, ctx->nblk, ctx->st));
  CKL(scft::launch_free_energy_finalize(ctx->partial, ctx->nblk, ctx->batch, ctx->M, ctx->Q,
                                        ctx->fe5, ctx->st));
  return SCFT_OK;
}

// Synchronise the stream and check the device error word that the pipelined
// kernels set when a bounded wait gives up.
int sync_check(scft_ctx *ctx) {
  CK(cudaStreamSynchronize(ctx->st));
  unsigned w = 0;
  CK(cudaMemcpy(&w, ctx->dev_err, sizeof(w), cudaMemcpyDeviceToHost));
  if (w) {
    cudaMemset(ctx->dev_err, 0, sizeof(unsigned));
    return scft_fail(ctx, SCFT_ERR_CUDA,
                     "a pipelined kernel timed out waiting for its bulk copies (error word " +
                         std::to_string(w) + "); results of that launch are invalid");
  }
  return SCFT_OK;
}

int read_fe(scft_ctx *ctx, double *out5) {
  CK(cudaMemcpyAsync(out5, ctx->fe5, sizeof(double) * 5 * ctx->batch, cudaMemcpyDeviceToHost,
                     ctx->st));
  if (int rc = sync_check(ctx)) return rc;
  for (int i = 0; i < 5 * ctx->batch; ++i)
    if (!isfinite(out5[i])) return scft_fail(ctx, SCFT_ERR_NOT_FINITE, "free energy is not finite");
  return SCFT_OK;
}

int pre_mix(scft_ctx *ctx) {
  int rc;
  if ((rc = average(ctx, ctx->wa))) return rc;   // cuda_scft.cu:170
  if ((rc = average(ctx, ctx->wb))) return rc;   // :172
  return get_conc(ctx);                          // :174
}

int iterate_once(scft_ctx *ctx) {
  int rc = pre_mix(ctx);
  if (rc) return rc;
  return mix(ctx);                               // :182
}

void free_all(scft_ctx *ctx) {
  cudaFree(ctx->wa); cudaFree(ctx->wb); cudaFree(ctx->pha); cudaFree(ctx->phb);
  for (int i = 0; i < 4; ++i) cudaFree(ctx->q[i]);
  cudaFree(ctx->qint);
  for (int i = 0; i < 2; ++i) cudaFree(ctx->W[i]);
  for (int i = 0; i < 4; ++i) cudaFree(ctx->tmp[i]);
  if (ctx->march_exec) cudaGraphExecDestroy(ctx->march_exec);
  ctx->march_exec = nullptr;
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  if (ctx->st2) cudaStreamDestroy(ctx->st2);
  cudaFree(ctx->partial); cudaFree(ctx->sum); cudaFree(ctx->Q); cudaFree(ctx->ffl);
  cudaFree(ctx->fe5); cudaFree(ctx->tables); cudaFree(ctx->dev_err);
  cudaFree(ctx->res); cudaFree(ctx->rpartial); cudaFree(ctx->gram); cudaFree(ctx->and_a);
  cudaFree(ctx->and_lam); cudaFree(ctx->target); cudaFree(ctx->dgain);
  cudaFree(ctx->shift_alpha);
  scft_internal_adjoint_free(ctx);
  for (float *h : ctx->hist_u) cudaFree(h);
  for (float *h : ctx->hist_d) cudaFree(h);
  ctx->hist_u.clear();
  ctx->hist_d.clear();
  cudaFree(ctx->wprev);
  for (cudaEvent_t e : ctx->prof_events) cudaEventDestroy(e);
  ctx->prof_events.clear();
  if (ctx->st) cudaStreamDestroy(ctx->st);
}

}  // namespace

// Schedule autotuner: every legal combination of chain schedule (lockstep /
// two streams), x+y fusion and column-pass kernel (one tile per CTA /
// persistent pipelined) is captured and timed on the real march phase (three
// replays after a warm-up, minimum taken); the fastest stays.  The fields are
// whatever the context holds (timings do not depend on their values).
int autotune(scft_ctx *ctx) {
  bool has_fast_col = false;   // the persistent column kernel exists in FP32 only
  for (size_t i = 1; i < ctx->passes.size(); ++i)
    has_fast_col |= ctx->rbytes == 4 && ctx->passes[i].use_fast != 0;
  const bool can_xy = ctx->fuse_xy;
  const bool can_fs = (ctx->p.flags & SCFT_FLAG_NO_FUSED_STEPS) == 0 && ctx->passes.size() == 3;
  int rc;
  if ((rc = boltzmann(ctx, SCFT_FIELD_WA, ctx->st))) return rc;
  if ((rc = boltzmann(ctx, SCFT_FIELD_WB, ctx->st))) return rc;
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  double best = 1e300;
  bool best_two = ctx->two_streams, best_xy = ctx->fuse_xy, best_pipe = ctx->use_pipe;
  bool best_fs = ctx->fuse_steps;
  for (int two = 0; two < 2; ++two)
    for (int xy = 0; xy < (can_xy ? 2 : 1); ++xy)
      for (int pipe = 0; pipe < (has_fast_col ? 2 : 1); ++pipe)
      for (int fs = 0; fs < (can_fs ? 2 : 1); ++fs) {
        // fused step pairs run only on two-stream chains and the plain column
        // kernels (with the x+y plane, or with three register-resident passes)
        if (fs && (!two || pipe)) continue;
        ctx->two_streams = two;
        ctx->fuse_xy = can_xy && xy;
        ctx->use_pipe = pipe;
        ctx->fuse_steps = fs;
        if (fs && !fused_possible(ctx)) continue;
        if (ctx->march_exec) cudaGraphExecDestroy(ctx->march_exec);
        ctx->march_exec = nullptr;
        if ((rc = march_phase_graph(ctx))) break;   // capture + warm-up
        double ms = 1e300;
        for (int r = 0; r < 3 && !rc; ++r) {
          cudaEventRecord(a, ctx->st);
          rc = march_phase_graph(ctx);
          cudaEventRecord(b, ctx->st);
          cudaEventSynchronize(b);
          float f = 0.f;
          cudaEventElapsedTime(&f, a, b);
          if (f < ms) ms = f;
        }
        if (rc) break;
        if (ms < best) {
          best = ms;
          best_two = two;
          best_xy = ctx->fuse_xy;
          best_pipe = pipe;
          best_fs = fs;
        }
      }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  ctx->two_streams = best_two;
  ctx->fuse_xy = best_xy;
  ctx->use_pipe = best_pipe;
  ctx->fuse_steps = best_fs;
  if (ctx->march_exec) cudaGraphExecDestroy(ctx->march_exec);
  ctx->march_exec = nullptr;
  ctx->tuned_ms = best;
  ctx->launches = 0;
  return sync_check(ctx);
}

// Hooks for the group graph (group.cu).
int scft_internal_pre_mix(scft_ctx *ctx) { return pre_mix(ctx); }

// Pieces of pre_mix for the group's batched march (group.cu): everything
// before the march phase (average_value x3, the Boltzmann factors), the march
// phase alone, and everything after it (Q, phi).
int scft_internal_pre_march(scft_ctx *ctx) {
  int rc;
  if ((rc = average(ctx, ctx->wa))) return rc;   // cuda_scft.cu:170
  if ((rc = average(ctx, ctx->wb))) return rc;   // :172
  if ((rc = average(ctx, ctx->wa))) return rc;   // getConc, :71
  if ((rc = boltzmann(ctx, SCFT_FIELD_WA, ctx->st))) return rc;
  return boltzmann(ctx, SCFT_FIELD_WB, ctx->st);
}
int scft_internal_march(scft_ctx *ctx) { return march_phase_graph(ctx); }
int scft_internal_post_march(scft_ctx *ctx) {
  const int rc = with_real(ctx, [&](auto r) { return q_and_phi<decltype(r)>(ctx); });
  ctx->have_conc = rc == SCFT_OK;
  return rc;
}

namespace {
// The two march chains of getConc as march_phase runs them.
void chain_segs(const scft_ctx *ctx, int chain, Seg out[2]) {
  if (chain == 0) {
    out[0] = {SCFT_Q_A, SCFT_FIELD_WA, -1, 0, ctx->NsA, 1};
    out[1] = {SCFT_Q_B, SCFT_FIELD_WB, SCFT_Q_A, ctx->NsA, ctx->dNsB, 1};
  } else {
    out[0] = {SCFT_Q_CB, SCFT_FIELD_WB, -1, 0, ctx->dNsB, -1};
    out[1] = {SCFT_Q_CA, SCFT_FIELD_WA, SCFT_Q_CB, 0, ctx->NsA, -1};
  }
}
}  // namespace

// Contour step t (1-based) of march chain `chain` in lockstep order (the
// run_chains schedule): whether the chain still marches at t, the slice it
// reads and the slice it writes, the Boltzmann factor, and the segment whose
// boundary slice must be set before the step (-1: none).  FP32 contexts.
int scft_internal_chain_step(const scft_ctx *ctx, int chain, int t, int *active,
                             const float **src, float **dst, const float **W, int *seg_start) {
  Seg sg[2];
  chain_segs(ctx, chain, sg);
  *active = 0;
  *seg_start = -1;
  int k = 0, it = t;
  if (t < 1 || t > sg[0].ns + sg[1].ns) return SCFT_OK;
  while (it > sg[k].ns) it -= sg[k++].ns;
  const Seg &s = sg[k];
  const long long M = ctx->M;
  float *q = static_cast<float *>(ctx->q[s.qi]);
  const int d = s.sign > 0 ? it : s.ns - it;
  *active = 1;
  *dst = q + (long long)d * M;
  *src = q + (long long)(s.sign > 0 ? d - 1 : d + 1) * M;
  *W = static_cast<const float *>(ctx->W[s.wf]);
  if (it == 1) *seg_start = k;
  return SCFT_OK;
}

// initilize_q / qInt copy of segment `seg` of chain `chain` (seg_boundary).
int scft_internal_seg_boundary(scft_ctx *ctx, int chain, int seg, cudaStream_t st) {
  Seg sg[2];
  chain_segs(ctx, chain, sg);
  return seg_boundary<float>(ctx, sg[seg], st);
}
int scft_internal_mix(scft_ctx *ctx) { return mix(ctx); }
int scft_internal_get_conc(scft_ctx *ctx) { return get_conc(ctx); }

namespace {
template <typename R>
int filter_impl(scft_ctx *ctx, const R *in, long long in_bs, R *out, long long out_bs,
                const R *pre, const R *post, long long w_bs, int nb, int deriv_pass, R *s0,
                R *s1, cudaStream_t st) {
  const long long M = ctx->M;
  const int np = (int)ctx->passes.size();
  for (int pi = 0; pi < np; ++pi) {
    scft::PassSet<R> p;
    memset(&p, 0, sizeof(p));
    p.nset = 1;
    p.batch = nb;
    p.w_bs = w_bs;
    p.in[0] = pi == 0 ? in : ((pi - 1) & 1 ? s1 : s0);
    p.in_bs[0] = pi == 0 ? in_bs : M;
    p.out[0] = pi == np - 1 ? out : (pi & 1 ? s1 : s0);
    p.out_bs[0] = pi == np - 1 ? out_bs : M;
    p.pre[0] = pi == 0 ? pre : nullptr;
    p.post[0] = pi == np - 1 ? post : nullptr;
    AxisPlan ap = ctx->passes[pi];
    if (pi == deriv_pass) ap.gain = ctx->dgain_pass[pi];
    int rc = launch_set<R>(ctx, ap, p, st);
    if (rc) return rc;
  }
  return SCFT_OK;
}
}  // namespace

int scft_internal_filter(scft_ctx *ctx, const void *in, long long in_bs, void *out,
                         long long out_bs, const void *pre, const void *post, long long w_bs,
                         int nb, int deriv_pass, void *s0, void *s1, cudaStream_t st) {
  return with_real(ctx, [&](auto r) {
    using R = decltype(r);
    return filter_impl<R>(ctx, (const R *)in, in_bs, (R *)out, out_bs, (const R *)pre,
                          (const R *)post, w_bs, nb, deriv_pass, (R *)s0, (R *)s1, st);
  });
}

int scft_fail(scft_ctx *ctx, int status, const std::string &msg) {
  if (ctx) ctx->err = msg;
  else g_create_err = msg;
  return status;
}

extern "C" {

int scft_params_default(scft_params *p) {
  if (!p) return SCFT_ERR_INVALID_ARG;
  memset(p, 0, sizeof(*p));
  p->nx = p->ny = p->nz = 32;
  p->lx = p->ly = p->lz = 4.0;
  p->hAB = 20.0;
  p->fA = 0.5;
  p->ds0 = 0.01;
  p->batch = 1;
  p->precision = SCFT_PREC_FP64;
  p->wopt = 0.05;
  p->wcmp = 0.10;
  p->mixing = SCFT_MIX_SIMPLE;
  p->anderson_history = 20;
  p->anderson_lambda = 0.5;
  p->anderson_start = 1.0;
  p->device = 0;
  return SCFT_OK;
}

int scft_grid_supported(int nx, int ny, int nz) {
  return axis_ok(nx, false) && axis_ok(ny, true) && axis_ok(nz, true);
}

const char *scft_strerror(int s) {
  switch (s) {
    case SCFT_OK: return "ok";
    case SCFT_ERR_INVALID_ARG: return "invalid argument";
    case SCFT_ERR_UNSUPPORTED: return "unsupported grid or option";
    case SCFT_ERR_CUDA: return "CUDA error";
    case SCFT_ERR_NO_MEMORY: return "out of memory";
    case SCFT_ERR_NOT_FINITE: return "non-finite value";
    case SCFT_ERR_IO: return "I/O error";
    case SCFT_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

const char *scft_last_error(const scft_ctx *ctx) {
  return ctx ? ctx->err.c_str() : g_create_err.c_str();
}

int scft_create(const scft_params *pin, scft_ctx **out) {
  scft_ctx *ctx = nullptr;
  if (!pin || !out) return scft_fail(nullptr, SCFT_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  const scft_params &p = *pin;
  for (size_t i = 0; i < sizeof(p.reserved) / sizeof(p.reserved[0]); ++i)
    if (p.reserved[i]) return scft_fail(nullptr, SCFT_ERR_INVALID_ARG, "reserved fields must be 0");
  if (p.flags & ~(SCFT_FLAG_NO_GRAPH | SCFT_FLAG_PIPE | SCFT_FLAG_TWO_STREAMS |
                  SCFT_FLAG_LOCKSTEP | SCFT_FLAG_NO_XY | SCFT_FLAG_AUTOTUNE |
                  SCFT_FLAG_NO_FUSED_STEPS | SCFT_FLAG_SIMPSON | SCFT_FLAG_PIN_TRANSLATION))
    return scft_fail(nullptr, SCFT_ERR_INVALID_ARG, "bad flags");
  if (!(p.lx > 0 && p.ly > 0 && p.lz > 0 && p.ds0 > 0 && p.fA >= 0 && p.fA <= 1 && p.batch >= 1))
    return scft_fail(nullptr, SCFT_ERR_INVALID_ARG, "bad box, ds0, fA or batch");
  if (p.precision != SCFT_PREC_FP64 && p.precision != SCFT_PREC_FP32 &&
      p.precision != SCFT_PREC_DF)
    return scft_fail(nullptr, SCFT_ERR_INVALID_ARG, "bad precision");
  if (p.mixing < SCFT_MIX_SIMPLE || p.mixing > SCFT_MIX_CONSTRAINED_EX)
    return scft_fail(nullptr, SCFT_ERR_INVALID_ARG, "bad mixing mode");
  if (p.mixing == SCFT_MIX_ANDERSON &&
      (p.anderson_history < 1 || p.anderson_history > 32 || !(p.anderson_lambda > 0)))
    return scft_fail(nullptr, SCFT_ERR_INVALID_ARG,
                     "Anderson history must be 1..32 and its step positive");
  if ((p.flags & SCFT_FLAG_PIN_TRANSLATION) && p.mixing != SCFT_MIX_ANDERSON)
    return scft_fail(nullptr, SCFT_ERR_INVALID_ARG,
                     "SCFT_FLAG_PIN_TRANSLATION acts on Anderson updates: it needs SCFT_MIX_ANDERSON");
  if (!scft_grid_supported(p.nx, p.ny, p.nz))
    return scft_fail(nullptr, SCFT_ERR_UNSUPPORTED,
                     "grid unsupported: Nx must be even, Ny/Nz even or 1, each <= 4096 with "
                     "prime factors <= 61");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return scft_fail(nullptr, SCFT_ERR_NO_DEVICE, "no CUDA device");
  if (p.device < 0 || p.device >= ndev)
    return scft_fail(nullptr, SCFT_ERR_NO_DEVICE, "bad device ordinal");
  if (cudaSetDevice(p.device) != cudaSuccess)
    return scft_fail(nullptr, SCFT_ERR_NO_DEVICE, "cudaSetDevice failed");

  ctx = new scft_ctx();
  ctx->p = p;
  ctx->M = (long long)p.nx * p.ny * p.nz;
  ctx->batch = p.batch;
  ctx->rbytes = p.precision == SCFT_PREC_FP32 ? 4 : 8;
  ctx->rkind = p.precision == SCFT_PREC_FP32 ? kRealF32
               : p.precision == SCFT_PREC_DF ? kRealDF : kRealF64;
  ctx->NsA = (int)(p.fA / p.ds0 + 1.0e-8);            // init_cuda.cu:330
  ctx->dNsB = (int)((1 - p.fA) / p.ds0 + 1.0e-8);     // init_cuda.cu:329,331
  ctx->q_ns[SCFT_Q_A] = ctx->q_ns[SCFT_Q_CA] = ctx->NsA;
  ctx->q_ns[SCFT_Q_B] = ctx->q_ns[SCFT_Q_CB] = ctx->dNsB;
  const long long M = ctx->M, B = ctx->batch;
  const size_t rb = ctx->rbytes;

  auto fail = [&](int st, const std::string &m) {
    std::string msg = m;
    free_all(ctx);
    delete ctx;
    return scft_fail(nullptr, st, msg);
  };
  ctx->use_graph = (p.flags & SCFT_FLAG_NO_GRAPH) == 0;
  ctx->use_pipe = (p.flags & SCFT_FLAG_PIPE) != 0;
  // Two forked chains beat shared lockstep launches once a pass fills the GPU
  // (measured, FP32 unfused: +16% at 128^3, +9% at 256^3, -8% at 64^3; FP64:
  // 25.2 against 32.1 ms per iteration at 64^3, even at 128^3).  With fused
  // step pairs they win at every size (below).
  const long long pts = (long long)p.nx * p.ny * p.nz * p.batch;
  ctx->two_streams = (p.flags & SCFT_FLAG_TWO_STREAMS) != 0 ||
                     ((p.flags & SCFT_FLAG_LOCKSTEP) == 0 &&
                      (pts >= (1LL << 20) ||
                       (p.precision == SCFT_PREC_FP64 && pts >= (1LL << 18))));
  if (cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->st2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess)
    return fail(SCFT_ERR_CUDA, "stream creation failed");
  if (scft::line_filter_prepare() != cudaSuccess || scft::fast_line_prepare() != cudaSuccess)
    return fail(SCFT_ERR_CUDA, "kernel attribute set-up failed");

  auto alloc = [&](void **ptr, size_t bytes) {
    if (cudaMalloc(ptr, bytes) != cudaSuccess) { *ptr = nullptr; return false; }
    return cudaMemset(*ptr, 0, bytes) == cudaSuccess;
  };
  bool ok = alloc((void **)&ctx->wa, 8 * M * B) && alloc((void **)&ctx->wb, 8 * M * B) &&
            alloc((void **)&ctx->pha, 8 * M * B) && alloc((void **)&ctx->phb, 8 * M * B);
  for (int i = 0; ok && i < 4; ++i) ok = alloc(&ctx->q[i], rb * M * B * (ctx->q_ns[i] + 1));
  ok = ok && alloc(&ctx->qint, rb * M * B) && alloc(&ctx->W[0], rb * M * B) &&
       alloc(&ctx->W[1], rb * M * B);
  for (int i = 0; ok && i < 4; ++i) ok = alloc(&ctx->tmp[i], rb * M * B);
  ctx->nblk = scft::reduce_blocks(M);
  ok = ok && alloc((void **)&ctx->partial, 8 * B * 3 * ctx->nblk) &&
       alloc((void **)&ctx->sum, 8 * B) && alloc((void **)&ctx->Q, 8 * B) &&
       alloc((void **)&ctx->ffl, 8 * B) && alloc((void **)&ctx->fe5, 8 * 5 * B) &&
       alloc((void **)&ctx->dev_err, sizeof(unsigned)) &&
       alloc((void **)&ctx->res, 8 * 4 * B) &&   // [b][2] residual norms + [b][2] means
       alloc((void **)&ctx->rpartial, 8 * B * scft::anderson_max_slots() * ctx->nblk);
  if (ok && p.mixing == SCFT_MIX_ANDERSON) {
    ctx->m1 = p.anderson_history + 1;
    ctx->hist_u.assign(ctx->m1, nullptr);
    ctx->hist_d.assign(ctx->m1, nullptr);
    for (int j = 0; ok && j < ctx->m1; ++j)
      ok = alloc((void **)&ctx->hist_u[j], 8 * 2 * M * B) &&
           alloc((void **)&ctx->hist_d[j], 8 * 2 * M * B);
    ok = ok && alloc((void **)&ctx->gram, 8 * B * ctx->m1 * ctx->m1) &&
         alloc((void **)&ctx->and_a, 8 * B * ctx->m1) && alloc((void **)&ctx->and_lam, 8 * 2 * B);
    if (p.flags & SCFT_FLAG_PIN_TRANSLATION)
      ok = ok && alloc((void **)&ctx->shift_alpha, 8 * 3 * B) &&
           alloc((void **)&ctx->wprev, 8 * 2 * M * B);
  }
  if (!ok) {
    cudaGetLastError();
    return fail(SCFT_ERR_NO_MEMORY, "device allocation failed");
  }

  // ---- per-axis spectral tables (init_cuda.cu:394-428, split per axis)
  const int dims[3] = {p.nx, p.ny, p.nz};
  const double lens[3] = {p.lx, p.ly, p.lz};
  std::vector<int> axes;
  for (int a = 0; a < 3; ++a)
    if (dims[a] != 1) axes.push_back(a);
  size_t tab_bytes = 0;
  for (int a : axes) tab_bytes += (size_t)dims[a] * 3 * rb + 256;
  if (!alloc(&ctx->tables, tab_bytes)) return fail(SCFT_ERR_NO_MEMORY, "table allocation failed");
  std::vector<unsigned char> host(tab_bytes, 0);
  size_t off = 0;
  for (size_t ai = 0; ai < axes.size(); ++ai) {
    const int a = axes[ai];
    const int n = dims[a];
    AxisPlan ap;
    memset(&ap, 0, sizeof(ap));
    ap.n = n;
    radix_plan(n, ap.fac, &ap.nfac);
    if (a == 0) {        // x: rows of Nx, contiguous
      ap.s_n = 1; ap.s_pair = p.nx; ap.s_outer = 0; ap.n_real = p.ny * p.nz; ap.n_outer = 1;
      ap.n_fast = 1;
    } else if (a == 1) { // y: stride Nx, pairs along x, outer z
      ap.s_n = p.nx; ap.s_pair = 1; ap.s_outer = (long long)p.nx * p.ny; ap.n_real = p.nx;
      ap.n_outer = p.nz; ap.n_fast = 0;
    } else {             // z: stride Nx*Ny, pairs along x, outer y
      ap.s_n = (long long)p.nx * p.ny; ap.s_pair = 1; ap.s_outer = p.nx; ap.n_real = p.nx;
      ap.n_outer = p.ny; ap.n_fast = 0;
    }
    const int n_pairs = (ap.n_real + 1) / 2;
    int tl = (int)(65536 / (4 * (size_t)n * rb));
    if (tl > 32) tl = 32;
    if (tl < 1) tl = 1;
    if (tl > n_pairs) tl = n_pairs;
    ap.tl = tl;
    ap.use_fast = scft::fast_line_supported(ap, rb) ? 1 : 0;
    // Column passes (y, z) tile 64 columns of one row.  When Nx is not a
    // multiple of 64 they run over flattened columns instead: z over the whole
    // (x, y) plane (contiguous), y over (x, z) (row c / Nx, outer stride
    // Nx*Ny).  That gives grids such as 32^3 and 48^3 register passes on every
    // axis (and with them the fused step pairs).
    if (a != 0 && !ap.use_fast && p.nx % 4 == 0) {
      AxisPlan flat = ap;
      flat.n_outer = 1;
      if (a == 2) {
        flat.n_real = p.nx * p.ny;
        flat.s_outer = 0;
      } else {
        flat.n_real = p.nx * p.nz;
        flat.s_outer = (long long)p.nx * p.ny;
        flat.flat_nx = p.nx;
      }
      if (scft::fast_line_supported(flat, rb)) {
        ap = flat;
        ap.use_fast = 1;
      }
    }
    if (ctx->rkind == kRealDF && (!ap.use_fast || (n != 32 && n != 64 && n != 128)))
      return fail(SCFT_ERR_UNSUPPORTED,
                  "double-float propagation needs register-resident passes: Nx of 32, 64 "
                  "or 128, Ny and Nz of 1, 32, 64 or 128, Ny*Nz a multiple of 64, "
                  "Nx*Nz and Nx*Ny multiples of 64 when Nx is 32");
    if (scft::line_filter_smem_bytes(ap, rb) > (size_t)scft::kLineSmemMax)
      return fail(SCFT_ERR_UNSUPPORTED, "line too long for shared memory");
    // twiddles exp(-2 pi i m / n); the gains are filled by upload_gains
    const size_t tw_off = off, g_off = off + (size_t)n * 2 * rb;
    for (int m = 0; m < n; ++m) {
      const double ang = -2.0 * M_PI * (double)m / (double)n;
      const double c = cos(ang), s = sin(ang);
      if (rb == 4) {
        float *t = reinterpret_cast<float *>(&host[tw_off]);
        t[2 * m] = (float)c; t[2 * m + 1] = (float)s;
      } else if (ctx->rkind == kRealDF) {
        scft::dfloat *t = reinterpret_cast<scft::dfloat *>(&host[tw_off]);
        t[2 * m] = scft::dfloat(c); t[2 * m + 1] = scft::dfloat(s);
      } else {
        double *t = reinterpret_cast<double *>(&host[tw_off]);
        t[2 * m] = c; t[2 * m + 1] = s;
      }
    }
    ap.twiddle = static_cast<unsigned char *>(ctx->tables) + tw_off;
    ap.gain = static_cast<unsigned char *>(ctx->tables) + g_off;
    off += (size_t)n * 3 * rb;
    off = (off + 255) & ~(size_t)255;
    ctx->pass_axis[ctx->passes.size()] = a;
    ctx->passes.push_back(ap);
  }
  // x and y both as their own passes (no length-1 axis among them) and small
  // enough for a shared-memory plane: fuse them
  ctx->fuse_xy = rb == 4 && (p.flags & SCFT_FLAG_NO_XY) == 0 && ctx->passes.size() >= 2 &&
                 axes[0] == 0 && axes[1] == 1 &&
                 scft::xy_fusable(ctx->passes[0], ctx->passes[1]);
  // fused step pairs need three passes: the x+y plane kernel and a
  // register-resident z pass, or three register-resident axis passes
  ctx->fuse_steps = (p.flags & SCFT_FLAG_NO_FUSED_STEPS) == 0;
  ctx->fuse_steps = fused_possible(ctx);
  // With fused step pairs the two-stream chains win at every size the plane
  // kernel takes (measured per SCF iteration: 64^3 1.12 ms against 1.27 ms
  // lockstep, 128^3 4.46 ms against 5.79 ms).
  if (ctx->fuse_steps && (p.flags & SCFT_FLAG_LOCKSTEP) == 0) ctx->two_streams = true;
  if (cudaMemcpy(ctx->tables, host.data(), tab_bytes, cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(SCFT_ERR_CUDA, "table upload failed");
  if (upload_gains(ctx)) return fail(SCFT_ERR_CUDA, "gain table upload failed: " + ctx->err);
  if (cudaDeviceSynchronize() != cudaSuccess) return fail(SCFT_ERR_CUDA, "set-up failed");
  ctx->err = "no error";
  if (p.flags & SCFT_FLAG_AUTOTUNE) {
    const int rc = autotune(ctx);
    if (rc) return fail(rc, "autotune: " + ctx->err);
  }
  *out = ctx;
  return SCFT_OK;
}

void scft_destroy(scft_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->p.device);
  if (ctx->st) cudaStreamSynchronize(ctx->st);
  free_all(ctx);
  delete ctx;
}

int scft_get_ns(const scft_ctx *ctx, int *NsA, int *dNsB) {
  if (!ctx || !NsA || !dNsB) return SCFT_ERR_INVALID_ARG;
  *NsA = ctx->NsA;
  *dNsB = ctx->dNsB;
  return SCFT_OK;
}

static double *field_ptr(scft_ctx *ctx, int f) {
  switch (f) {
    case SCFT_FIELD_WA: return ctx->wa;
    case SCFT_FIELD_WB: return ctx->wb;
    case SCFT_FIELD_PHA: return ctx->pha;
    case SCFT_FIELD_PHB: return ctx->phb;
    default: return nullptr;
  }
}

int scft_set_field(scft_ctx *ctx, int field, const double *src) {
  if (!ctx) return SCFT_ERR_INVALID_ARG;
  double *d = field_ptr(ctx, field);
  if (!d || !src) return scft_fail(ctx, SCFT_ERR_INVALID_ARG, "bad field or null pointer");
  CK(cudaMemcpyAsync(d, src, sizeof(double) * ctx->M * ctx->batch, cudaMemcpyHostToDevice, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  if (field == SCFT_FIELD_WA || field == SCFT_FIELD_WB) ctx->and_count = 0;  // new fields, new history
  return SCFT_OK;
}

int scft_get_field(scft_ctx *ctx, int field, double *dst) {
  if (!ctx) return SCFT_ERR_INVALID_ARG;
  double *d = field_ptr(ctx, field);
  if (!d || !dst) return scft_fail(ctx, SCFT_ERR_INVALID_ARG, "bad field or null pointer");
  CK(cudaMemcpyAsync(dst, d, sizeof(double) * ctx->M * ctx->batch, cudaMemcpyDeviceToHost, ctx->st));
  return sync_check(ctx);
}

int scft_average_value(scft_ctx *ctx, int field) {
  if (!ctx) return SCFT_ERR_INVALID_ARG;
  if (field != SCFT_FIELD_WA && field != SCFT_FIELD_WB)
    return scft_fail(ctx, SCFT_ERR_INVALID_ARG, "average_value applies to wa or wb");
  return average(ctx, field_ptr(ctx, field));
}

int scft_sov_dif_fft(scft_ctx *ctx, int q, int w_field, int ns, int sign) {
  if (!ctx) return SCFT_ERR_INVALID_ARG;
  if (q < 0 || q > 3 || (w_field != SCFT_FIELD_WA && w_field != SCFT_FIELD_WB) ||
      (sign != 1 && sign != -1) || ns < 0 || ns > ctx->q_ns[q])
    return scft_fail(ctx, SCFT_ERR_INVALID_ARG, "bad propagator, field, sign or ns");
  return march(ctx, q, w_field, ns, sign);
}

int scft_set_qint(scft_ctx *ctx, int q, int s) {
  if (!ctx) return SCFT_ERR_INVALID_ARG;
  if (q > 3 || (q >= 0 && (s < 0 || s > ctx->q_ns[q])))
    return scft_fail(ctx, SCFT_ERR_INVALID_ARG, "bad propagator or slice");
  return set_qint(ctx, q, s);
}

int scft_get_q(scft_ctx *ctx, int q, int s, double *dst) {
  if (!ctx) return SCFT_ERR_INVALID_ARG;
  if (q < 0 || q > 3 || s < 0 || s > ctx->q_ns[q] || !dst)
    return scft_fail(ctx, SCFT_ERR_INVALID_ARG, "bad propagator, slice or pointer");
  const long long M = ctx->M;
  const long long qbs = (long long)(ctx->q_ns[q] + 1) * M;
  // stage through the (FP64-sized) phi scratch: cast on the device, then copy
  double *stage = nullptr;
  CK(cudaMallocAsync((void **)&stage, sizeof(double) * M * ctx->batch, ctx->st));
  int rc = with_real(ctx, [&](auto r) {
    using R = decltype(r);
    CKL(scft::launch_cast_slice<R>(stage, M, static_cast<R *>(ctx->q[q]) + (long long)s * M, qbs,
                                   M, ctx->batch, ctx->st));
    return SCFT_OK;
  });
  if (rc) {
    cudaFreeAsync(stage, ctx->st);
    return rc;
  }
  CK(cudaMemcpyAsync(dst, stage, sizeof(double) * M * ctx->batch, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaFreeAsync(stage, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return SCFT_OK;
}

int scft_get_conc(scft_ctx *ctx) {
  if (!ctx) return SCFT_ERR_INVALID_ARG;
  return get_conc(ctx);
}

int scft_get_Q(scft_ctx *ctx, double *dst) {
  if (!ctx || !dst) return SCFT_ERR_INVALID_ARG;
  CK(cudaMemcpyAsync(dst, ctx->Q, sizeof(double) * ctx->batch, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return SCFT_OK;
}

int scft_phi_w(scft_ctx *ctx) {
  if (!ctx) return SCFT_ERR_INVALID_ARG;
  return mix(ctx);
}

int scft_set_target(scft_ctx *ctx, const double *pha_target) {
  if (!ctx || !pha_target) return SCFT_ERR_INVALID_ARG;
  CK(cudaSetDevice(ctx->p.device));
  const size_t bytes = sizeof(double) * ctx->M * ctx->batch;
  if (!ctx->target) CK(cudaMalloc((void **)&ctx->target, bytes));
  CK(cudaMemcpyAsync(ctx->target, pha_target, bytes, cudaMemcpyHostToDevice, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return SCFT_OK;
}

int scft_phi_w_constrained(scft_ctx *ctx, int ex, double lambda) {
  if (!ctx) return SCFT_ERR_INVALID_ARG;
  if (!ctx->target) return scft_fail(ctx, SCFT_ERR_INVALID_ARG, "no target field set");
  CKL(scft::launch_phi_w_constrained(ctx->wa, ctx->wb, ctx->pha, ctx->phb, ctx->target,
                                     ctx->p.hAB, lambda, ex != 0, ctx->M, ctx->batch, ctx->st));
  return SCFT_OK;
}

int scft_free_energy(scft_ctx *ctx, double *out5) {
  if (!ctx || !out5) return SCFT_ERR_INVALID_ARG;
  int rc = free_energy_dev(ctx);
  if (rc) return rc;
  return read_fe(ctx, out5);
}

int scft_iterate(scft_ctx *ctx, int n_iter, double *out5) {
  if (!ctx || n_iter < 0) return SCFT_ERR_INVALID_ARG;
  for (int it = 0; it < n_iter; ++it) {
    int rc = iterate_once(ctx);
    if (rc) return rc;
  }
  if (out5) {
    int rc = free_energy_dev(ctx);
    if (rc) return rc;
    return read_fe(ctx, out5);
  }
  return SCFT_OK;
}

int scft_set_metrics_file(scft_ctx *ctx, const char *path) {
  if (!ctx) return SCFT_ERR_INVALID_ARG;
  ctx->metrics_path = path ? path : "";
  return SCFT_OK;
}

namespace {
// A JSON number (round-trip precision), or null for NaN/Inf (not JSON numbers).
std::string json_num(double v) {
  if (!std::isfinite(v)) return "null";
  char b[32];
  snprintf(b, sizeof b, "%.17g", v);
  return b;
}

// One JSON line per instance for a progress report (scft_set_metrics_file);
// `first` is the global number of the context's instance 0 (its shard's
// offset when instances are split over several devices).
int write_metrics(scft_ctx *ctx, int iter, const double *fe, double elapsed_s, int first) {
  std::vector<double> mx(ctx->batch), rms(ctx->batch);
  int rc = scft_get_residual(ctx, mx.data(), rms.data());
  if (rc) return rc;
  FILE *fp = fopen(ctx->metrics_path.c_str(), "a");
  if (!fp) return scft_fail(ctx, SCFT_ERR_IO, "cannot append to " + ctx->metrics_path);
  static const char *keys[5] = {"F", "F_AB", "F_W", "F_S", "inCompMax"};
  for (int i = 0; i < ctx->batch; ++i) {
    std::string line = "{\"iteration\":" + std::to_string(iter) +
                       ",\"instance\":" + std::to_string(first + i);
    for (int k = 0; k < 5; ++k) line += std::string(",\"") + keys[k] + "\":" + json_num(fe[5 * i + k]);
    line += ",\"residual_max\":" + json_num(mx[i]) + ",\"residual_rms\":" + json_num(rms[i]) +
            ",\"elapsed_s\":" + json_num(elapsed_s) + "}\n";
    fputs(line.c_str(), fp);
  }
  return fclose(fp) == 0 ? SCFT_OK : scft_fail(ctx, SCFT_ERR_IO, "write " + ctx->metrics_path);
}
}  // namespace

// init_cuda.cu:312: cufft_info->batch = Num_SCFT / GPU_N.  The reference's
// integer split: every device gets the same count, and the last
// Num_SCFT % GPU_N instances (read from their phi_<i>.dat) are never run.
int scft_shard_plan(int num_scft, int gpu_n, int *batch_per_gpu, int *not_run) {
  if (!batch_per_gpu || gpu_n < 1 || gpu_n > SCFT_MAX_SHARDS || num_scft < 1)
    return scft_fail(nullptr, SCFT_ERR_INVALID_ARG, "bad instance or device count");
  if (num_scft < gpu_n)
    return scft_fail(nullptr, SCFT_ERR_INVALID_ARG,
                     "fewer instances than devices: the split would leave a device with none");
  *batch_per_gpu = num_scft / gpu_n;
  if (not_run) *not_run = num_scft % gpu_n;
  return SCFT_OK;
}

// Free (cuda_scft.cu:140-269) over instances split across devices
// (init_cuda.cu:312): shard g holds global instances g*batch .. g*batch +
// batch-1.  Each iteration is enqueued on every shard's own stream before any
// shard is waited for, so the devices run concurrently; nothing is exchanged
// between them.  Progress lines and pha_<i>.dat files come out in the
// reference's order (shard by shard, instance by instance) with its numbering.
int scft_free_shards(scft_ctx *const *ctxs, int n, int max_it, int aver_it, const char *outdir) {
  if (!ctxs || n < 1 || n > SCFT_MAX_SHARDS || max_it < 0 || aver_it < 1)
    return scft_fail(nullptr, SCFT_ERR_INVALID_ARG, "bad shard list or iteration counts");
  for (int g = 0; g < n; ++g)
    if (!ctxs[g] || ctxs[g]->batch != ctxs[0]->batch)
      return scft_fail(nullptr, SCFT_ERR_INVALID_ARG,
                       "every shard needs a context with the same instance count");
  const int batch = ctxs[0]->batch;
  std::vector<double> fe(5 * (size_t)batch);
  const auto t0 = std::chrono::steady_clock::now();
  int iter = 0;
  do {                                   // cuda_scft.cu:167-253
    iter = iter + 1;
    for (int g = 0; g < n; ++g) {
      scft_ctx *ctx = ctxs[g];
      if (cudaSetDevice(ctx->p.device) != cudaSuccess)
        return scft_fail(ctx, SCFT_ERR_CUDA, "cudaSetDevice failed");
      if (int rc = iterate_once(ctx)) return rc;
    }
    if (iter % aver_it != 0) continue;
    for (int g = 0; g < n; ++g) {
      scft_ctx *ctx = ctxs[g];
      cudaSetDevice(ctx->p.device);
      int rc;
      if ((rc = free_energy_dev(ctx))) return rc;
      if ((rc = read_fe(ctx, fe.data()))) return rc;
      for (int i = 0; i < batch; ++i)
        printf("GPU %d batch %d: %5d : %.8e, %.8e, %.8e,%.8e, %.8e\n", g, i, iter, fe[5 * i + 0],
               fe[5 * i + 1], fe[5 * i + 2], fe[5 * i + 3], fe[5 * i + 4]);
      fflush(stdout);
      if (!ctx->metrics_path.empty()) {
        const double el =
            std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if ((rc = write_metrics(ctx, iter, fe.data(), el, g * batch))) return rc;
      }
    }
    if (outdir && iter % (aver_it * 10) == 0) {
      for (int g = 0; g < n; ++g) {
        cudaSetDevice(ctxs[g]->p.device);
        for (int i = 0; i < batch; ++i) {
          std::string path =
              std::string(outdir) + "/pha_" + std::to_string(g * batch + i + 1) + ".dat";
          if (int rc = scft_write_pha_dat(ctxs[g], path.c_str(), i)) return rc;
        }
      }
    }
  } while (iter < max_it);
  for (int g = 0; g < n; ++g) {
    cudaSetDevice(ctxs[g]->p.device);
    if (int rc = sync_check(ctxs[g])) return rc;
  }
  return SCFT_OK;
}

int scft_free(scft_ctx *ctx, int max_it, int aver_it, const char *outdir) {
  if (!ctx || max_it < 0 || aver_it < 1) return SCFT_ERR_INVALID_ARG;
  return scft_free_shards(&ctx, 1, max_it, aver_it, outdir);
}

int scft_synchronize(scft_ctx *ctx) {
  if (!ctx) return SCFT_ERR_INVALID_ARG;
  return sync_check(ctx);
}

int scft_set_box(scft_ctx *ctx, double lx, double ly, double lz) {
  if (!ctx) return SCFT_ERR_INVALID_ARG;
  if (!(lx > 0 && ly > 0 && lz > 0)) return scft_fail(ctx, SCFT_ERR_INVALID_ARG, "bad box");
  CK(cudaSetDevice(ctx->p.device));
  // the tables are read by every pass launch (the captured graphs included,
  // also a group's): no launch of this context may be in flight
  CK(cudaDeviceSynchronize());
  ctx->p.lx = lx;
  ctx->p.ly = ly;
  ctx->p.lz = lz;
  ctx->and_count = 0;   // the history belongs to the old operator
  ctx->have_conc = false;   // the stored propagators belong to the old box
  return upload_gains(ctx);
}

int scft_copy_q_reference_layout(scft_ctx *ctx, int q, double *dst_device) {
  if (!ctx || !dst_device || q < 0 || q > 3)
    return scft_fail(ctx, SCFT_ERR_INVALID_ARG, "bad propagator or null pointer");
  CK(cudaSetDevice(ctx->p.device));
  int rc = with_real(ctx, [&](auto r) {
    using R = decltype(r);
    CKL(scft::launch_q_to_reference_layout<R>(static_cast<const R *>(ctx->q[q]), ctx->q_ns[q],
                                              ctx->M, ctx->batch, dst_device, ctx->st));
    return SCFT_OK;
  });
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->st));
  return SCFT_OK;
}

int scft_selftest_bounded_wait(int device, double seconds, int *timed_out) {
  scft_ctx *ctx = nullptr;   // errors go to the create-time message
  if (!timed_out || !(seconds > 0) || seconds > 10)
    return scft_fail(nullptr, SCFT_ERR_INVALID_ARG, "timed_out null or seconds not in (0, 10]");
  *timed_out = 0;
  int clk_khz = 0;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, device) != cudaSuccess)
    return scft_fail(nullptr, SCFT_ERR_NO_DEVICE, "no such device");
  unsigned *err = nullptr;
  CK(cudaMalloc(&err, sizeof(unsigned)));
  unsigned h = 0;
  cudaError_t e = cudaMemset(err, 0, sizeof(unsigned));
  if (e == cudaSuccess)
    e = scft::launch_wait_selftest(err, (long long)(seconds * clk_khz * 1e3), nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(&h, err, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(err);
  if (e != cudaSuccess) return scft_fail(nullptr, SCFT_ERR_CUDA, cudaGetErrorString(e));
  *timed_out = (h & 4u) != 0;
  return SCFT_OK;
}

int scft_field_device_ptr(scft_ctx *ctx, int field, double **dptr) {
  if (!ctx || !dptr) return SCFT_ERR_INVALID_ARG;
  double *p = field_ptr(ctx, field);
  if (!p) return scft_fail(ctx, SCFT_ERR_INVALID_ARG, "bad field");
  *dptr = p;
  return SCFT_OK;
}

int scft_get_stream(scft_ctx *ctx, void **stream) {
  if (!ctx || !stream) return SCFT_ERR_INVALID_ARG;
  *stream = ctx->st;
  return SCFT_OK;
}

int scft_get_box(const scft_ctx *ctx, double *L3) {
  if (!ctx || !L3) return SCFT_ERR_INVALID_ARG;
  L3[0] = ctx->p.lx;
  L3[1] = ctx->p.ly;
  L3[2] = ctx->p.lz;
  return SCFT_OK;
}

int scft_get_schedule(const scft_ctx *ctx, int *flags, double *march_ms) {
  if (!ctx) return SCFT_ERR_INVALID_ARG;
  if (flags)
    *flags = (ctx->two_streams ? SCFT_FLAG_TWO_STREAMS : SCFT_FLAG_LOCKSTEP) |
             (ctx->fuse_xy ? 0 : SCFT_FLAG_NO_XY) | (ctx->use_pipe ? SCFT_FLAG_PIPE : 0) |
             (ctx->fuse_steps && ctx->two_streams ? 0 : SCFT_FLAG_NO_FUSED_STEPS);
  if (march_ms) *march_ms = ctx->tuned_ms;
  return SCFT_OK;
}

int scft_get_residual(scft_ctx *ctx, double *err_max, double *err_rms) {
  if (!ctx) return SCFT_ERR_INVALID_ARG;
  std::vector<double> e(2 * ctx->batch);
  CK(cudaMemcpyAsync(e.data(), ctx->res, sizeof(double) * e.size(), cudaMemcpyDeviceToHost,
                     ctx->st));
  if (int rc = sync_check(ctx)) return rc;
  for (int b = 0; b < ctx->batch; ++b) {
    if (err_max) err_max[b] = e[2 * b];
    if (err_rms) err_rms[b] = e[2 * b + 1];
  }
  return SCFT_OK;
}

int scft_converge(scft_ctx *ctx, double tol, int max_it, int *iters, double *out5) {
  if (!ctx || max_it < 0 || !(tol > 0)) return SCFT_ERR_INVALID_ARG;
  NvtxRange range("scft converge");
  std::vector<double> e(ctx->batch);
  int it = 0;
  while (it < max_it) {
    int rc = iterate_once(ctx);
    if (rc) return rc;
    ++it;
    if ((rc = scft_get_residual(ctx, e.data(), nullptr))) return rc;
    bool done = true;
    for (double v : e) {
      if (!std::isfinite(v)) {
        if (iters) *iters = it;
        return scft_fail(ctx, SCFT_ERR_NOT_FINITE, "residual is not finite (diverged)");
      }
      if (!(v < tol)) done = false;
    }
    if (done) break;
  }
  if (iters) *iters = it;
  if (out5) {
    int rc = free_energy_dev(ctx);
    if (rc) return rc;
    return read_fe(ctx, out5);
  }
  return SCFT_OK;
}

int scft_copy_fields(scft_ctx *dst, const scft_ctx *src) {
  if (!dst || !src) return SCFT_ERR_INVALID_ARG;
  scft_ctx *ctx = dst;   // errors are reported on the destination
  if (dst->M != src->M || dst->batch != src->batch)
    return scft_fail(dst, SCFT_ERR_INVALID_ARG, "contexts differ in grid or batch");
  const size_t bytes = sizeof(double) * dst->M * dst->batch;
  CK(cudaStreamSynchronize(src->st));
  CK(cudaMemcpyAsync(dst->wa, src->wa, bytes, cudaMemcpyDeviceToDevice, dst->st));
  CK(cudaMemcpyAsync(dst->wb, src->wb, bytes, cudaMemcpyDeviceToDevice, dst->st));
  CK(cudaMemcpyAsync(dst->pha, src->pha, bytes, cudaMemcpyDeviceToDevice, dst->st));
  CK(cudaMemcpyAsync(dst->phb, src->phb, bytes, cudaMemcpyDeviceToDevice, dst->st));
  // Anderson restarts on the copied fields: a history whose residuals came
  // from FP32 propagation slows an FP64 polish down (measured: 185 polish
  // iterations with the carried history against 76 with a fresh one).
  dst->and_count = 0;
  return sync_check(dst);
}

long long scft_launch_count(const scft_ctx *ctx) { return ctx ? ctx->launches : -1; }

int scft_time_iterations(scft_ctx *ctx, int n_iter, double *ms) {
  if (!ctx || !ms || n_iter < 0) return SCFT_ERR_INVALID_ARG;
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  CK(cudaEventRecord(a, ctx->st));
  int rc = SCFT_OK;
  for (int it = 0; it < n_iter && rc == SCFT_OK; ++it) rc = iterate_once(ctx);
  cudaEventRecord(b, ctx->st);
  cudaEventSynchronize(b);
  float f = 0.f;
  cudaEventElapsedTime(&f, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = f;
  return rc;
}

int scft_profile_enable(scft_ctx *ctx, int enable) {
  if (!ctx || enable < 0) return SCFT_ERR_INVALID_ARG;
  ctx->profiling = enable > 0;
  if (enable > 0) return prof_reserve(ctx, 2 * (size_t)enable);
  return SCFT_OK;
}

int scft_profile_read(scft_ctx *ctx, double *march_ms, long long *n_marches,
                      double *point_steps) {
  if (!ctx || !march_ms || !n_marches || !point_steps) return SCFT_ERR_INVALID_ARG;
  CK(cudaStreamSynchronize(ctx->st));
  double tot = 0.0;
  for (size_t i = 0; i + 1 < ctx->prof_used; i += 2) {
    float f = 0.f;
    CK(cudaEventElapsedTime(&f, ctx->prof_events[i], ctx->prof_events[i + 1]));
    tot += f;
  }
  *march_ms = tot;
  *n_marches = (long long)(ctx->prof_used / 2);
  *point_steps = ctx->prof_point_steps;
  ctx->prof_used = 0;
  ctx->prof_point_steps = 0.0;
  return SCFT_OK;
}

}  // extern "C"
