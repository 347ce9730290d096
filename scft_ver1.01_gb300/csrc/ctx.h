// Internal state behind the opaque scft_ctx of include/scft_capi.h.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <string>
#include <vector>

#include "scft_capi.h"
#include "kernels.h"

struct scft_ctx {
  scft_params p;
  int NsA = 0, dNsB = 0;
  long long M = 0;
  int batch = 0;
  int rbytes = 8;               // sizeof working real (4 or 8)
  int rkind = 1;                // working real: kRealF32, kRealF64 or kRealDF
  cudaStream_t st = nullptr;    // the context's stream (every launch)
  bool use_graph = true;        // march phase replayed as a CUDA graph
  bool capturing = false;       // inside a group graph capture: launch directly
  bool use_pipe = false;        // persistent pipelined column passes (opt-in)
  bool two_streams = false;     // march chains on two forked streams instead of lockstep
  bool fuse_xy = false;         // x and y passes fused into one plane kernel (FP32)
  bool fuse_steps = false;      // two-stream chains run fused step pairs (one launch per step)
  double tuned_ms = 0.0;        // march-phase time of the autotuned schedule
  cudaStream_t st2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  unsigned *dev_err = nullptr;  // device error word (bounded-wait timeouts)
  cudaGraphExec_t march_exec = nullptr;
  long long march_nodes = 0;    // kernel launches inside the graph
  std::string err;
  std::string metrics_path;     // JSON-lines progress reports of scft_free ("" = off)
  long long launches = 0;

  // FP64 fields [batch][M]
  double *wa = nullptr, *wb = nullptr, *pha = nullptr, *phb = nullptr;
  // propagators [batch][ns_q+1][M] in the working precision
  void *q[4] = {nullptr, nullptr, nullptr, nullptr};
  int q_ns[4] = {0, 0, 0, 0};
  void *qint = nullptr;         // [batch][M]
  void *W[2] = {nullptr, nullptr};   // Boltzmann factors of wa / wb [batch][M]
  void *tmp[4] = {nullptr, nullptr, nullptr, nullptr};  // pass intermediates, 2 per chain
  // reductions
  int nblk = 1;
  double *partial = nullptr;    // [batch][3][nblk]
  double *sum = nullptr, *Q = nullptr, *ffl = nullptr, *fe5 = nullptr;
  // residual and Anderson mixing
  double *res = nullptr;          // [batch][2]: residual max|d|, rms(d)
  double *rpartial = nullptr;     // [batch][33][nblk] reduction partials
  int m1 = 0;                     // Anderson ring slots (history + 1)
  // ring of [batch][2][M] double-float pairs (hi, lo floats, 8 bytes a
  // value): u = w + anderson_lambda d and the mean-free residual d
  std::vector<float *> hist_u, hist_d;
  double *wprev = nullptr;        // [batch][2][M] pre-update fields (SCFT_FLAG_PIN_TRANSLATION)
  double *gram = nullptr;         // [batch][m1][m1]
  double *and_a = nullptr;        // [batch][m1] slot weights
  double *and_lam = nullptr;      // [2][batch]: step, mode (1 Anderson, 0 simple)
  double *shift_alpha = nullptr;  // [batch][3] rigid-shift coefficients (SCFT_FLAG_PIN_TRANSLATION)
  long long and_count = 0;        // iterations stored in the ring
  double *target = nullptr;       // [batch][M] target phiA of the constrained updates
  // spectral tables (twiddles + gains of each pass), device
  void *tables = nullptr;
  std::vector<scft::AxisPlan> passes;
  int pass_axis[3] = {0, 0, 0};       // grid axis (0 x, 1 y, 2 z) of each pass
  // box derivatives: per pass the gain times d(-ds k^2)/dL of its axis,
  // and for length-1 axes (no pass) the constant d(-ds k^2)/dL
  void *dgain = nullptr;
  const void *dgain_pass[3] = {nullptr, nullptr, nullptr};
  double unit_c[3] = {0.0, 0.0, 0.0};
  struct AdjointState *adj = nullptr;   // adjoint / stress work buffers (lazy)
  bool have_conc = false;       // propagators, W and Q of a getConc at the current box
  // per-march event timing
  bool profiling = false;
  std::vector<cudaEvent_t> prof_events;   // pairs, grown on demand
  size_t prof_used = 0;
  double prof_point_steps = 0.0;
};

// The working real type of the propagators (float, double or the
// double-float pair), and a dispatch on it: with_real(ctx, f) calls f(R{}).
constexpr int kRealF32 = 0, kRealF64 = 1, kRealDF = 2;
template <typename F> int with_real(const scft_ctx *ctx, F &&f) {
  if (ctx->rkind == kRealF32) return f(float{});
  if (ctx->rkind == kRealDF) return f(scft::dfloat{});
  return f(double{});
}

// NVTX range for profilers (a no-op unless a tool is attached).
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

// Set ctx->err and return status.
int scft_fail(scft_ctx *ctx, int status, const std::string &msg);

// One application of the step operator's diffusion part to nb slices:
// out = post * K (pre * in), K = the per-axis line filters of the context
// (x, y, z passes, no plane fusion).  deriv_pass >= 0 swaps that pass's gain
// for its box-derivative gain.  s0 and s1 hold the intermediates (nb slices
// of M each); in, out, s0 and s1 must not overlap.  Working precision.
int scft_internal_filter(scft_ctx *ctx, const void *in, long long in_bs, void *out,
                         long long out_bs, const void *pre, const void *post, long long w_bs,
                         int nb, int deriv_pass, void *s0, void *s1, cudaStream_t st);
// getConc (cuda_scft.cu:61-138) on the context's fields.
int scft_internal_get_conc(scft_ctx *ctx);
// Releases the adjoint work buffers (adjoint.cu).
void scft_internal_adjoint_free(scft_ctx *ctx);
