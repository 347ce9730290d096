// Host-side launchers of the SCFT kernels (all run on one CUDA stream each).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "dfloat.cuh"

namespace scft {

// One per-axis pass of the separable diffusion operator exp(-k^2 ds):
// every line along the axis is transformed, multiplied by the real, even
// gain g[k] (= exp(-ds*k^2)/N, the reference's kxyzdz factor split per axis),
// and transformed back.  Two real lines are packed as the real and imaginary
// parts of one complex line; because g is real and even the two lines do not
// mix.  Geometry of the real lines of one instance:
//   element (outer o, real line r, position n) at  o*s_outer + r*s_pair + n*s_n
struct AxisPlan {
  int n;                 // line length
  int nfac;              // radix plan (Stockham stages), product == n
  int fac[24];
  long long s_n, s_pair, s_outer;
  int n_real;            // real lines per outer group (paired 2 by 2)
  int n_outer;           // outer groups per instance
  int n_fast;            // 1: consecutive threads walk n (contiguous lines)
  int flat_nx;           // column passes: 0, or the row length when the columns run over a
                         // flattened (row, outer) index: column c sits at
                         // (c / flat_nx) * s_outer + c % flat_nx (n_outer 1)
  int tl;                // complex lines per CTA tile
  int use_fast;          // FP32 register-resident kernel (k_fast.cu) handles this pass
  const void *twiddle;   // device: n complex, exp(-2*pi*i*m/n), working precision
  const void *gain;      // device: n reals, working precision
};

// One pass over up to kMaxSet independent propagators at once (the lockstep
// march chains): set k reads in[k] (+ b*in_bs), multiplies by pre[k], filters,
// multiplies by post[k] and writes out[k] (+ b*out_bs), for every instance b.
constexpr int kMaxSet = 2;
// One line set of a batched pass over several contexts (a group's lockstep
// march, FP32): the set's buffers (one instance each) and gain tables.
struct PassDesc {
  const float *in;
  float *out;
  const float *pre, *post;   // Boltzmann factor on load / on store, or null
  const float *gain;         // the set's gain table of this pass's axis (x for a plane pass)
  const float *gain_y;       // x+y plane passes: the y axis's gain table
};
template <typename R> struct PassSet {
  const R *in[kMaxSet];
  R *out[kMaxSet];
  const R *pre[kMaxSet];
  const R *post[kMaxSet];
  long long in_bs[kMaxSet], out_bs[kMaxSet];
  long long w_bs;
  int nset;
  int batch;
  unsigned *err;   // device error word (bounded-wait timeouts), may be null for non-pipelined kernels
  // fused step pairs only (launch_zz / launch_xyxy): where the finished
  // propagator slice goes; `out` then receives the next step's intermediate
  R *qout[kMaxSet];
  long long qout_bs[kMaxSet];
  // FP32 per-axis and x+y plane passes: when set, line set blockIdx.z takes
  // its buffers and gains from desc[blockIdx.z] (nset 1, batch = sets)
  const PassDesc *desc;
};

// Register-resident pass (k_fast.cu): n in {32, 64, 128, 256} (FP32) or
// {32, 64, 128} (FP64), and n_real a multiple of 64.
bool fast_line_supported(const AxisPlan &ap, size_t real_bytes = 4);
// Fused x+y pass over whole z-planes (k_fast.cu): Nx, Ny in {64, 128}.
bool xy_fusable(const AxisPlan &apx, const AxisPlan &apy);
cudaError_t launch_xy(const AxisPlan &apx, const AxisPlan &apy, const PassSet<float> &ps,
                      cudaStream_t st);
cudaError_t fast_line_prepare();
// x+y passes of 256 x 256 planes (k_plane256.cu): a cluster of two CTAs per
// plane, the y lines read across the pair through distributed shared memory;
// launch_xy / launch_xyxy dispatch here for such planes.
bool plane256_fusable(const AxisPlan &apx, const AxisPlan &apy);
cudaError_t plane256_prepare();
cudaError_t launch_xy256(const AxisPlan &apx, const AxisPlan &apy, const PassSet<float> &ps,
                         cudaStream_t st);
cudaError_t launch_xyxy256(const AxisPlan &apx, const AxisPlan &apy, const PassSet<float> &ps,
                           cudaStream_t st);
// bounded-wait self-test: sets bit 4 of *err after `limit` clocks
cudaError_t launch_wait_selftest(unsigned *err, long long limit, cudaStream_t st);
cudaError_t launch_fast_line(const AxisPlan &ap, const PassSet<float> &ps, cudaStream_t st);
cudaError_t launch_fast_line(const AxisPlan &ap, const PassSet<double> &ps, cudaStream_t st);
cudaError_t launch_fast_line(const AxisPlan &ap, const PassSet<dfloat> &ps, cudaStream_t st);
// Fused step pairs.  The axis filters commute, so consecutive contour steps
// can run their passes in alternating order (x+y then z, z then x+y); the
// end of one step and the start of the next are then the same pass type and
// run as one kernel: qout = post * K_a(in), out = K_a(post * qout), with
// K_a the z filter (launch_zz) or the x+y filters (launch_xyxy).
cudaError_t launch_zz(const AxisPlan &ap, const PassSet<float> &ps, cudaStream_t st);
cudaError_t launch_zz(const AxisPlan &ap, const PassSet<double> &ps, cudaStream_t st);
cudaError_t launch_zz(const AxisPlan &ap, const PassSet<dfloat> &ps, cudaStream_t st);
// the same on x lines (rows contiguous), for grids without the x+y plane
cudaError_t launch_xx(const AxisPlan &ap, const PassSet<float> &ps, cudaStream_t st);
cudaError_t launch_xx(const AxisPlan &ap, const PassSet<double> &ps, cudaStream_t st);
cudaError_t launch_xx(const AxisPlan &ap, const PassSet<dfloat> &ps, cudaStream_t st);
cudaError_t launch_xyxy(const AxisPlan &apx, const AxisPlan &apy, const PassSet<float> &ps,
                        cudaStream_t st);

// Generic mixed-radix Stockham line filter (any n whose prime factors are
// <= 61).  in/out may not alias.  pre multiplies the input, post the output
// (elementwise, indexed like one instance's grid); either may be null.
template <typename R>
cudaError_t launch_line_filter(const AxisPlan &ap, const R *in, long long in_bstride, R *out,
                               long long out_bstride, const R *pre, const R *post,
                               long long w_bstride, int batch, cudaStream_t st);
// The same over n line sets described by desc[0..n) (FP32, device memory).
cudaError_t launch_line_filter_desc(const AxisPlan &ap, const PassDesc *desc, int n,
                                    cudaStream_t st);

size_t line_filter_smem_bytes(const AxisPlan &ap, size_t real_bytes);
constexpr int kLineSmemMax = 200 * 1024;
cudaError_t line_filter_prepare();

// ---- residual and Anderson mixing (k_anderson.cu) ----
int anderson_max_slots();
// residual of phi_w's update (err[b][2] = max, rms); optionally stores
// u = w + lam_u d and d into a history slot (hu, hd: [b][2][M] double-float
// pairs), copies w to wprev ([b][2][M] FP64) and/or applies the simple step
// w += wopt*d (4 kernels)
cudaError_t launch_residual(double *wa, double *wb, const double *pha, const double *phb,
                            double hAB, double wcmp, double wopt, long long M, int batch,
                            void *hu, void *hd, double lam_u, double *wprev, double *partial,
                            int nblk, double *err, cudaStream_t st);
// Gram row <d_c, d_j> (double-float ring slots) into the FP64 ring matrix
// (2 kernels)
cudaError_t launch_gram_row(const void *dc, const void *const *dj, const int *slots, int n,
                            int c, int m1, long long M, int batch, double *partial, int nblk,
                            double *G, cudaStream_t st);
// weights a[b][m1], step lam[b] and mode lam[batch + b] (1 Anderson, 0 simple)
cudaError_t launch_anderson_solve(const double *G, const double *err, int c, int hist, int m1,
                                  double start, double lambda, double wopt, int batch,
                                  double *a, double *lam, cudaStream_t st);
// The update w0 -> (wa, wb) without its component along the rigid shifts of
// w0 ([b][2][M], central differences, periodic): three kernels; partial holds
// batch*9*nblk doubles, alpha batch*3.
cudaError_t launch_remove_translation(double *wa, double *wb, const double *w0, int nx, int ny,
                                     int nz, int batch, double *partial, int nblk,
                                     double *alpha, cudaStream_t st);
// w_new = sum_k a_k u_k over the listed ring slots (Anderson step) or
// w + lam d_c (simple step), per instance as the solve decided
cudaError_t launch_anderson_update(double *wa, double *wb, const void *const *hu, const void *dc,
                                   const int *idx, int n, const double *a, const double *lam,
                                   int m1, long long M, int batch, cudaStream_t st);

// ---- field kernels (k_fields.cu) ----
// W = exp(-w*ds2) in precision R, for batch*M points (w is FP64).
template <typename R>
cudaError_t launch_boltzmann(const double *w, R *W, long long n, double ds2, cudaStream_t st);
template <typename R>
cudaError_t launch_fill(R *x, long long n, R v, long long bstride, int batch, cudaStream_t st);
// dst[b*dst_bstride + i] = src[b*src_bstride + i], i < M
template <typename R>
cudaError_t launch_copy_slice(R *dst, long long dst_bstride, const R *src, long long src_bstride,
                              long long M, int batch, cudaStream_t st);
template <typename R>
cudaError_t launch_cast_slice(double *dst, long long dst_bstride, const R *src,
                              long long src_bstride, long long M, int batch, cudaStream_t st);

// Deterministic per-instance sums: partial[b*nblk+k] then finalize.
int reduce_blocks(long long M);
template <typename R>
cudaError_t launch_partial_sum(const R *x, long long bstride, long long M, int batch,
                               double *partial, int nblk, cudaStream_t st);
cudaError_t launch_finalize_sum(const double *partial, int nblk, int batch, double scale,
                                double *out, cudaStream_t st);
// data -= sum/M  (minus_average)
cudaError_t launch_minus_average(double *data, const double *sum, long long M, int batch,
                                 cudaStream_t st);
// Q = sum/M ; ffl = ds0/Q  (cal_ql + host lines of getConc)
cudaError_t launch_q_ffl(const double *sum, long long M, double ds0, int batch, double *Q,
                         double *ffl, cudaStream_t st);
// Weight of contour point s (0..n) of a block of n steps: the reference's
// trapezoid (1/2 at both ends, 1 inside; the n == 0 block has the single
// weight 1/2, cuda_aid.cu:87-107), or Simpson (1/3 rule; for odd n >= 3 the
// 3/8 rule over the last three steps; n == 1 stays trapezoid).
double contour_weight(int s, int n, bool simpson);
// The same weights in kernel form: interior points 1..m-1 take c_odd (odd s)
// or c_even (even s); up to five listed points take their own weight.
struct ContourWeights {
  int m, nspec;
  double c_odd, c_even;
  int s[5];
  double w[5];
};
ContourWeights contour_weights(int n, bool simpson);
// phi = ffl * contour sum of q*qc with the weights above (w_to_phi_go)
template <typename R>
cudaError_t launch_contour_phi(const R *q, const R *qc, int ns, long long M, int batch,
                               const double *ffl, double *phi, bool simpson, cudaStream_t st);
// simple mixing (phi_w); writes the residual max-norm partials if resid != null
cudaError_t launch_phi_w(double *wa, double *wb, const double *pha, const double *phb,
                         double hAB, double wopt, double wcmp, long long M, int batch,
                         cudaStream_t st);
// propagator [b][s][M] -> g[b][r][s] FP64 (the reference's layout)
template <typename R>
cudaError_t launch_q_to_reference_layout(const R *q, int ns, long long M, int batch, double *g,
                                         cudaStream_t st);
// phi_w_constrained (ex == 0) / phi_w_constrainedEx (ex != 0)
cudaError_t launch_phi_w_constrained(double *wa, double *wb, const double *pha, const double *phb,
                                     const double *target, double hAB, double lambda, int ex,
                                     long long M, int batch, cudaStream_t st);
// free energy partials: sums of hAB*pa*pb, wa*pa+wb*pb and max|1-pa-pb|
cudaError_t launch_free_energy_partials(const double *wa, const double *wb, const double *pha,
                                        const double *phb, double hAB, long long M, int batch,
                                        double *partial, int nblk, cudaStream_t st);
cudaError_t launch_free_energy_finalize(const double *partial, int nblk, int batch, long long M,
                                        const double *Q, double *out5, cudaStream_t st);

}  // namespace scft
