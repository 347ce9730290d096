/*
 * scft_capi.h -- C ABI of the GB300-native diblock-copolymer SCFT hot path.
 *
 * One opaque context = one GPU, `batch` independent SCFT instances of one
 * grid/parameter set (the reference's CUFFT_INFO + GPU_INFO, struct.h:19-125).
 * The reference's GPU_N split of the instances over devices is one context per
 * device (scft_shard_plan, scft_free_shards).  All entry points return an
 * SCFT_* status code and never exit the process; scft_last_error() gives the
 * message of the last failure on a context.
 *
 * Field arrays crossing this boundary are host float64 arrays laid out
 * [batch][Nz][Ny][Nx] (x fastest), the reference's ijk order
 * (init_cuda.cu:420-423, :509-512).  Propagators are stored on the device
 * contour-outer ([batch][s][Nz][Ny][Nx]) in the context's propagation
 * precision.
 *
 * Each declaration names the reference function it replaces (file:line).
 */
#ifndef SCFT_CAPI_H
#define SCFT_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define SCFT_OK 0
#define SCFT_ERR_INVALID_ARG 1    /* bad pointer, size, enum or parameter */
#define SCFT_ERR_UNSUPPORTED 2    /* grid the kernels do not handle (see scft_grid_supported) */
#define SCFT_ERR_CUDA 3           /* CUDA runtime error (message in scft_last_error) */
#define SCFT_ERR_NO_MEMORY 4      /* device or host allocation failed */
#define SCFT_ERR_NOT_FINITE 5     /* NaN/Inf detected in Q, F or the residual */
#define SCFT_ERR_IO 6             /* config / field file missing or malformed */
#define SCFT_ERR_NO_DEVICE 7      /* no CUDA device / bad ordinal */

/* ---- enums ---- */
#define SCFT_PREC_FP64 0          /* plain path: propagation and FFTs in FP64 */
#define SCFT_PREC_FP32 1          /* FP32 propagation, FP64 Q / contour sums / F / mixing */
#define SCFT_PREC_DF 2            /* propagation in double-float arithmetic (pairs of FP32
                                     numbers, ~48 significant bits) on the FP32 pipe, FP64
                                     elsewhere: FP64-level results faster than native FP64 on
                                     GB300; Nx of 64 or 128, Ny and Nz of 1, 32, 64 or 128,
                                     Ny*Nz a multiple of 64 */

#define SCFT_FIELD_WA 0
#define SCFT_FIELD_WB 1
#define SCFT_FIELD_PHA 2
#define SCFT_FIELD_PHB 3

/* propagators, named after the reference's buffers (struct.h:118-121) */
#define SCFT_Q_A 0                /* qa_cu : forward, A block, NsA+1 slices */
#define SCFT_Q_CB 1               /* qcb_cu: backward, B block, dNsB+1 slices */
#define SCFT_Q_B 2                /* qb_cu : forward, B block, dNsB+1 slices */
#define SCFT_Q_CA 3               /* qca_cu: backward, A block, NsA+1 slices */

#define SCFT_MIX_SIMPLE 0         /* phi_w (cuda_aid.cu:382-416) */
#define SCFT_MIX_ANDERSON 1       /* Anderson mixing on the phi_w residual (no reference counterpart) */
#define SCFT_MIX_CONSTRAINED 2    /* phi_w_constrained toward a target phiA (cuda_aid.cu:418-452) */
#define SCFT_MIX_CONSTRAINED_EX 3 /* phi_w_constrainedEx toward a target phiA (cuda_aid.cu:454-490) */

typedef struct scft_ctx scft_ctx;

/* Parameters: the ab.txt keys (init.cpp:86-92) plus the constants the
 * reference hard-codes (phi_w's wopt/wcmp, cuda_aid.cu:395-396) and the
 * options that have no reference counterpart (precision, mixing). */
typedef struct scft_params {
  int nx, ny, nz;           /* Nx, Ny, Nz: each even, or 1 for ny/nz */
  double lx, ly, lz;        /* box lengths in Rg */
  double hAB;               /* xN  (chi N) */
  double fA;                /* fa  (A fraction) */
  double ds0;               /* contour step */
  int batch;                /* independent instances on this device (batch) */
  int precision;            /* SCFT_PREC_* */
  double wopt;              /* simple-mixing step, reference 0.05 */
  double wcmp;              /* incompressibility weight, reference 0.10 */
  int mixing;               /* SCFT_MIX_* */
  int anderson_history;     /* Anderson history length m (1..32, e.g. 20) */
  double anderson_lambda;   /* Anderson step on the mixed residual */
  int device;               /* CUDA device ordinal */
  int flags;                /* SCFT_FLAG_* */
  double anderson_start;    /* simple mixing until the residual max-norm drops below this */
  double constraint_lambda; /* penalty weight of SCFT_MIX_CONSTRAINED (phi_w_constrained's lambda) */
  int reserved[4];          /* must be zero */
} scft_params;

/* flags */
#define SCFT_FLAG_NO_GRAPH 1      /* issue the march phase as plain launches, not a CUDA graph */
#define SCFT_FLAG_PIPE 2          /* persistent column passes with a cp.async.bulk staging ring
                                     (slower than the default one-tile-per-CTA kernel at 128^3) */
#define SCFT_FLAG_TWO_STREAMS 4   /* march chains on two forked streams (default when batch*M >= 2^20) */
#define SCFT_FLAG_LOCKSTEP 8      /* march chains in shared lockstep launches (default below 2^20 points) */
#define SCFT_FLAG_NO_XY 16        /* separate x and y passes instead of the fused plane kernel */
#define SCFT_FLAG_AUTOTUNE 32     /* time every legal schedule at creation and keep the fastest */
#define SCFT_FLAG_NO_FUSED_STEPS 64 /* two-stream chains: two launches per contour step instead of
                                       one fused kernel per step pair (k_zz / k_xyxy) */
#define SCFT_FLAG_PIN_TRANSLATION 256 /* Anderson mixing: remove from every field update its
                                     component along the fields' rigid shifts (central-
                                     difference gradients, least squares over both fields),
                                     so the iteration cannot drift along the translational
                                     zero mode and runs in different arithmetic from the
                                     same start reach the same, unshifted structure (no
                                     reference counterpart) */
#define SCFT_FLAG_SIMPSON 128     /* phi contour sums with Simpson weights instead of the
                                     reference's trapezoid (w_to_phi_go, cuda_aid.cu:87-107):
                                     composite 1/3 rule, the 3/8 rule over the last three steps
                                     of a block with an odd step count; the adjoint and the
                                     stress use the same weights */

/* Fill *p with the reference defaults (32^3, box 4, xN 20, fa 0.5,
 * ds0 0.01, batch 1, FP64, simple mixing wopt 0.05 wcmp 0.10). */
int scft_params_default(scft_params *p);

/* 1 if the grid is handled by this build's kernels, else 0. */
int scft_grid_supported(int nx, int ny, int nz);

/* Replaces init_cuda (init_cuda.cu:227-294) + initialize_cufft
 * (init_cuda.cu:296-546): selects the device, builds the per-axis spectral
 * tables (init_cuda.cu:394-428), NsA/dNsB (init_cuda.cu:330-331) and
 * allocates every device buffer.  Fields start at zero. */
int scft_create(const scft_params *p, scft_ctx **out);

/* Replaces finalize_cufft (init_cuda.cu:551-628).  NULL is ignored. */
void scft_destroy(scft_ctx *ctx);

/* Message of the last failure on ctx (or, when ctx is NULL, of the calling
 * host thread's last failed call without a context, e.g. scft_create).
 * Never NULL. */
const char *scft_last_error(const scft_ctx *ctx);
const char *scft_strerror(int status);

/* Contour discretisation (init_cuda.cu:330-331). */
int scft_get_ns(const scft_ctx *ctx, int *NsA, int *dNsB);

/* Host -> device copy of one field (the cudaMemcpy of wa/wb at
 * init_cuda.cu:509-512); src holds batch*M doubles. */
int scft_set_field(scft_ctx *ctx, int field, const double *src);
/* Device -> host copy of one field; dst holds batch*M doubles. */
int scft_get_field(scft_ctx *ctx, int field, double *dst);

/* Failure-detection self-test (no reference counterpart): runs the bounded
 * mbarrier wait of the pipelined kernels on a barrier nothing arrives at, for
 * `seconds` (at most 10) of SM clock, on `device`.  *timed_out = 1 when the
 * wait gave up and reported through the device error word (the kernel returns;
 * nothing traps or hangs).  Returns SCFT_OK while the device stays usable. */
int scft_selftest_bounded_wait(int device, double seconds, int *timed_out);

/* Zero-copy access (no reference counterpart; the reference hands out its
 * per-GPU device pointers through CUFFT_INFO, struct.h:94-121): the device
 * address of a field ([batch][M] FP64 on the context's device), valid until
 * scft_destroy, and the context's CUDA stream (a cudaStream_t).  Work a
 * caller does on the field must be ordered with that stream. */
int scft_field_device_ptr(scft_ctx *ctx, int field, double **dptr);
int scft_get_stream(scft_ctx *ctx, void **stream);

/* average_value (cuda_scft.cu:14-59): w -= <w> per instance, on
 * SCFT_FIELD_WA or SCFT_FIELD_WB. */
int scft_average_value(scft_ctx *ctx, int field);

/* sovDifFft (cuda_scft.cu:435-563): march propagator `q` (SCFT_Q_*) over
 * `ns` contour steps in the field `w_field` (SCFT_FIELD_WA/WB) from the
 * context's qInt buffer; sign=+1 fills slices 0..ns forward, sign=-1 fills
 * ns..0 backward.  ns must not exceed the propagator's slice count - 1. */
int scft_sov_dif_fft(scft_ctx *ctx, int q, int w_field, int ns, int sign);

/* qInt hand-offs of getConc: qInt_init (cuda_aid.cu:197-208) when q < 0,
 * otherwise qInt = slice s of propagator q (qa_to_qInt / qa_to_qInt2,
 * cuda_aid.cu:170-194). */
int scft_set_qint(scft_ctx *ctx, int q, int s);

/* Device -> host copy of slice s of propagator q, converted to FP64;
 * dst holds batch*M doubles. */
int scft_get_q(scft_ctx *ctx, int q, int s, double *dst);

/* The whole propagator q in the reference's own layout g[b][r][s] (s
 * fastest, FP64; cuda_aid.cu:237), written to caller-owned device memory of
 * batch*M*(ns_q+1) doubles by a tiled transpose.  The struct API keeps its
 * qa_cu/qb_cu/qca_cu/qcb_cu in this layout when built with
 * -DSCFT_COMPAT_FP64_LAYOUT. */
int scft_copy_q_reference_layout(scft_ctx *ctx, int q, double *dst_device);

/* getConc (cuda_scft.cu:61-138): average_value(wa), the four marches, Q and
 * the trapezoid contour sums giving pha/phb.  Stays on the device. */
int scft_get_conc(scft_ctx *ctx);

/* Q = ql/M per instance (cuda_scft.cu:118-126); dst holds batch doubles. */
int scft_get_Q(scft_ctx *ctx, double *dst);

/* phi_w simple mixing (cuda_aid.cu:382-416) with the context's wopt/wcmp. */
int scft_phi_w(scft_ctx *ctx);

/* The free-energy block of Free (cuda_scft.cu:188-221) on the current
 * fields: out5 holds batch*5 doubles {F, F_AB, F_W, F_S, inCompMax}. */
int scft_free_energy(scft_ctx *ctx, double *out5);

/* n_iter iterations of the body of Free (cuda_scft.cu:167-186):
 * average_value(wa), average_value(wb), getConc, then the field update of
 * the context's mixing mode.  No host round trip inside.  If out5 is not
 * NULL the free energy after the last iteration is written to it (batch*5
 * doubles, the reference's post-update convention). */
int scft_iterate(scft_ctx *ctx, int n_iter, double *out5);

/* Free (cuda_scft.cu:140-269): max_it iterations; every aver_it iterations
 * the reference's progress line "GPU %d batch %d: %5d : F, F_AB, F_W,F_S,
 * inCompMax" is printed to stdout, and every 10*aver_it iterations
 * pha_<i>.dat is written into `outdir` (NULL: no files).  Returns
 * SCFT_ERR_NOT_FINITE if F becomes NaN/Inf. */
int scft_free(scft_ctx *ctx, int max_it, int aver_it, const char *outdir);

/* ---- instances split over several devices (GPU_N / -gpu<i>) ---- */
#define SCFT_MAX_SHARDS 64
/* The reference's split of Num_SCFT instances over gpu_n devices
 * (init_cuda.cu:312, cufft_info->batch = Num_SCFT / GPU_N): every device gets
 * *batch_per_gpu instances; the last *not_run (= Num_SCFT % GPU_N, may be
 * NULL) are read but never run, as in the reference.  Host only.  Fewer
 * instances than devices is SCFT_ERR_INVALID_ARG. */
int scft_shard_plan(int num_scft, int gpu_n, int *batch_per_gpu, int *not_run);
/* Free (cuda_scft.cu:140-269) over n shards, one context per device (each
 * created with its device in scft_params.device and the same batch): shard g
 * holds global instances g*batch .. g*batch+batch-1.  Every iteration is
 * queued on all shards before any is waited for, so the devices run
 * concurrently; no data moves between them.  Progress lines read
 * "GPU <g> batch <i>" and files pha_<g*batch+i+1>.dat, the reference's
 * order and numbering.  scft_free(ctx, ...) is the n == 1 case. */
int scft_free_shards(scft_ctx *const *ctxs, int n, int max_it, int aver_it, const char *outdir);

/* Wait for all work queued on the context's stream. */
int scft_synchronize(scft_ctx *ctx);

/* The march schedule in use, as the SCFT_FLAG_* bits that select it
 * (TWO_STREAMS or LOCKSTEP, NO_XY, PIPE), and -- after SCFT_FLAG_AUTOTUNE --
 * the measured milliseconds of one march phase with it (else 0). */
int scft_get_schedule(const scft_ctx *ctx, int *flags, double *march_ms);

/* ---- convergence (no reference counterpart: the reference always runs
 * MaxIT iterations, cuda_scft.cu:253) ----
 * The residual is phi_w's update direction before the wopt step
 * (cuda_aid.cu:398-408): dA = xN phB + eta - wA - wcmp(1-phA-phB), dB likewise.
 * After each iteration the context holds err_max = max_r max(|dA|,|dB|) and
 * err_rms = sqrt(<dA^2+dB^2>/2), per instance. */
int scft_get_residual(scft_ctx *ctx, double *err_max, double *err_rms);

/* Iterate until every instance has err_max < tol or max_it iterations ran.
 * Mixing follows params.mixing: SCFT_MIX_SIMPLE is the reference's phi_w;
 * SCFT_MIX_ANDERSON uses simple mixing until err_max < anderson_start, then
 * Anderson mixing over the last anderson_history residuals (Gram matrix and
 * least squares in FP64, solved on the device).  *iters receives the
 * iterations run; out5 (batch*5 doubles, may be NULL) the free energy after
 * the last one.  Returns SCFT_ERR_NOT_FINITE on divergence. */
int scft_converge(scft_ctx *ctx, double tol, int max_it, int *iters, double *out5);

/* Device-to-device copy of wa, wb, pha, phb from src to dst (same grid and
 * batch; the contexts may differ in precision).  Used for an FP64 polish of
 * an FP32 solve. */
int scft_copy_fields(scft_ctx *dst, const scft_ctx *src);

/* Number of kernel launches issued on the context since creation (the
 * benchmark's gpu_launches evidence). */
long long scft_launch_count(const scft_ctx *ctx);

/* Timing hook of fft_test (cuda_scft.cu:411-425): run n_iter iterations as
 * scft_iterate does, bracketed by CUDA events recorded on the context's
 * stream; *ms receives the elapsed device time. */
int scft_time_iterations(scft_ctx *ctx, int n_iter, double *ms);

/* Per-march event timing (no reference counterpart).  While enabled, every
 * propagator march records an event pair on the context's stream;
 * scft_profile_read returns the summed device time of the marches, their
 * count and the grid-point x contour-step count they covered, then resets. */
int scft_profile_enable(scft_ctx *ctx, int enable);
int scft_profile_read(scft_ctx *ctx, double *march_ms, long long *n_marches,
                      double *point_steps);

/* ---- heterogeneous batched sweeps (no reference counterpart: the
 * reference's batch shares one grid and parameter set, init.cpp:86-94) ----
 * A group advances many contexts -- any mix of grids, xN, f, boxes, ds0 -- on
 * one device.  Each group iteration is one CUDA-graph launch that runs every
 * member's average_value x2 + getConc concurrently on the members' streams,
 * followed by each member's field update.  Members stay usable on their own;
 * do not use a member concurrently with its group. */
typedef struct scft_group scft_group;
int scft_group_create(scft_ctx *const *ctxs, int n, scft_group **out);
void scft_group_destroy(scft_group *g);
const char *scft_group_last_error(const scft_group *g);
int scft_group_iterate(scft_group *g, int n_iter);
int scft_group_time_iterations(scft_group *g, int n_iter, double *ms);
long long scft_group_launch_count(const scft_group *g);

/* ---- split step without device allocation ----
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * where they advance a propagator: a framework that owns all device memory
 * through its own pool, or loops that cannot afford cudaMalloc's implicit
 * synchronisation.
 * One FP32 split step q_out = W . IFFT[G . FFT[W . q_in]] / M (one contour
 * step of sovDifFft, cuda_scft.cu:467-491) for `batch` instances laid out
 * [batch][Nz][Ny][Nx]; q_in, W and q_out are caller-owned, 16-byte aligned
 * device buffers of batch*Nx*Ny*Nz floats (W: the Boltzmann factor
 * exp(-w*ds0/2)), enqueued on
 * `stream` (a cudaStream_t; NULL = default stream).  Scratch lives in a static
 * device array of this library: batch*Nx*Ny*Nz is limited to 2^21 points
 * and batch to 65535 (larger requests return SCFT_ERR_INVALID_ARG before
 * anything is enqueued), every GPU that loads the
 * library holds the array (~16 MB) until exit, and calls that overlap on the
 * GPU race on it.  The first call on a device looks up the array's address;
 * make it before any stream capture.  A returned error is this call's own
 * (an earlier, unrelated CUDA error does not fail it).  Never calls
 * cudaMalloc/cudaFree. */
int scft_split_step_noalloc(int nx, int ny, int nz, double lx, double ly, double lz, double ds0,
                            int batch, const float *q_in, const float *W, float *q_out,
                            void *stream);
/* Message of the last failed scft_split_step_noalloc call. */
const char *scft_noalloc_last_error(void);

/* ---- file formats (drop-in I/O) ---- */

/* Parse an ab.txt file (init.cpp:81-94) into *p (other fields default).
 * After the reference's seven lines, optional `key=value` lines (one per
 * line, no reference counterpart) set: mixing=simple|anderson, history=<m>,
 * lambda=<Anderson step>, start=<Anderson switch residual>, wopt=, wcmp=,
 * precision=fp32|fp64|df, Ns=<contour steps> (ds0 = 1/Ns); lines starting
 * with '#' are comments.  An unknown key or a bad value is SCFT_ERR_IO. */
int scft_read_ab_txt(const char *path, scft_params *p, int *intag);

/* ---- checkpoint / metrics (no reference counterpart) ---- */

/* Binary checkpoint for an exact resume (the reference's pha_<i>.dat keeps
 * 6 significant digits).  Holds the parameters and wa, wb, phiA, phiB of
 * every instance in FP64; with with_history != 0 and Anderson mixing also
 * the history ring (its double-float pairs as the device holds them), its
 * FP64 Gram matrix, the iteration count and lambda, so that a run resumed
 * with the same schedule repeats the uninterrupted run bit for bit.  Format
 * version 2 (files of version 1 are refused). */
int scft_save_checkpoint(scft_ctx *ctx, const char *path, int with_history);
/* Restore a checkpoint into a context of the same grid and batch
 * (SCFT_ERR_INVALID_ARG otherwise).  The history is restored only when the
 * precision, mixing, history length, Anderson lambda, box, xN, fA and ds0
 * also match; otherwise it restarts. */
int scft_load_checkpoint(scft_ctx *ctx, const char *path);

/* JSON-lines metrics: with a path set, every progress report of scft_free
 * also appends one line per instance,
 *   {"iteration":..,"instance":..,"F":..,"F_AB":..,"F_W":..,"F_S":..,
 *    "inCompMax":..,"residual_max":..,"residual_rms":..,"elapsed_s":..}
 * (residual: the mean-free max-norm and RMS of phi_w's update direction;
 * NaN or Inf is written as null).  NULL or "" turns it off.  The file is
 * opened for appending on each report. */
int scft_set_metrics_file(scft_ctx *ctx, const char *path);

/* Read phi_<idx>.dat (init_cuda.cu:435-456) for instance `inst` of the
 * context: pha/phb/wa/wb columns after two header lines.  The fields are
 * uploaded to the device. */
int scft_read_phi_dat(scft_ctx *ctx, const char *path, int inst);

/* Write pha_<idx>.dat (cuda_scft.cu:233-243) for instance `inst`. */
int scft_write_pha_dat(scft_ctx *ctx, const char *path, int inst);

/* Write phiA - phiB of instance `inst` as the ASCII STRUCTURED_POINTS file of
 * the reference's converter (vtk.c:54-76); `source` names the data in the
 * comment line (vtk.c:55). */
int scft_write_vtk(scft_ctx *ctx, const char *path, int inst, const char *source);

/* The reference's converter itself (vtk.c:4-81): pha_<i>.dat file -> VTK file. */
int scft_convert_pha_to_vtk(const char *pha_path, const char *vtk_path);

/* Target phiA field of the constrained updates ([batch][Nz][Ny][Nx] host
 * doubles, the reference's PhA_cu, cuda_aid.cu:418). */
int scft_set_target(scft_ctx *ctx, const double *pha_target);

/* One constrained field update on the current fields:
 * phi_w_constrained (cuda_aid.cu:418-452; constants wopt 0.05, wcmp 0.10,
 * penalty `lambda`) when ex == 0, phi_w_constrainedEx (cuda_aid.cu:454-490;
 * wopt 1.60, wcmp 0.50) when ex != 0. */
int scft_phi_w_constrained(scft_ctx *ctx, int ex, double lambda);

/* ---- derivatives (no reference counterpart) ----------------------------
 * F is the per-chain free energy of Free (cuda_scft.cu:190-221); the box
 * lengths lx, ly, lz enter only through the Gaussian factor exp(-ds k^2)
 * (init_cuda.cu:394-428), k_a = 2 pi m / L_a. */

/* Change the box (unit-cell) lengths: rewrites the spectral gain tables in
 * place.  The fields keep their grid values. */
int scft_set_box(scft_ctx *ctx, double lx, double ly, double lz);
/* The current box lengths (lx, ly, lz). */
int scft_get_box(const scft_ctx *ctx, double *L3);

/* SCFT stress of the propagators stored by the last getConc:
 * dF_dL[b*3 + a] = -d ln Q_b / dL_a at fixed fields (the partial derivative
 * of F at fixed w; at a saddle point it is the total dF/dL of the converged
 * free energy).  Spectral contraction of q and q+ with d exp(-ds k^2)/dL. */
int scft_stress(scft_ctx *ctx, double *dF_dL);

/* Reverse-mode adjoint (vector-Jacobian product) of getConc
 * (cuda_scft.cu:61-138) at the current fields: for the map
 * (wA, wB, box) -> (phiA, phiB, Q) and cotangents pha_bar, phb_bar
 * ([batch][M] host, null = 0) and Q_bar ([batch], null = 0), returns
 * wa_bar, wb_bar ([batch][M], null = not wanted) and L_bar ([batch][3],
 * null = skip the box terms).  The forward propagators are stored only every
 * `checkpoint_every` contour steps (0: ceil(sqrt(NsA + dNsB))) and recomputed
 * segment by segment during the reverse sweeps.  Includes getConc's mean
 * subtraction of wA. */
int scft_adjoint(scft_ctx *ctx, const double *pha_bar, const double *phb_bar,
                 const double *Q_bar, double *wa_bar, double *wb_bar, double *L_bar,
                 int checkpoint_every);

/* Propagator slices held by scft_adjoint for a checkpoint interval (0: the
 * default), and their bytes. */
int scft_adjoint_checkpoints(scft_ctx *ctx, int checkpoint_every, int *slices,
                             long long *bytes);

/* Unit-cell relaxation (batch == 1): converge the fields to max|dw| < tol_w
 * (scft_converge, at most max_inner iterations), take the stress, move the
 * box lengths selected by axes_mask (bit 0 x, 1 y, 2 z) by a Barzilai-Borwein
 * step on F*(L) (first step step0 * stress, at most 5% per step), and repeat
 * until max |stress| < tol_stress or max_outer rounds.  Returns the rounds,
 * the final stress [3] and the free energy [5] of the final fields; the box
 * is left at the relaxed lengths. */
int scft_relax_cell(scft_ctx *ctx, int axes_mask, double tol_w, double tol_stress,
                    int max_outer, int max_inner, double step0, int *outer_iters,
                    double *dF_dL, double *out5);

/* ---- cubic interpolating spline (spline.h / spline.c) -------------------
 * The Forsythe-Malcolm-Moler spline of the reference with its optional
 * known end slopes; same arguments and meaning, bit-identical results.  The
 * reference's own names are available from include/compat/spline.h. */

/* spline (spline.c:24-210): coefficients b, c, d (each n long) of the spline
 * through (x[i], y[i]); end1/end2 = 1 imposes slope1/slope2 at the ends,
 * 0 the default end conditions.  *iflag = 0 ok, 1 fewer than two knots,
 * 2 x not strictly increasing.  Returns SCFT_OK (or SCFT_ERR_INVALID_ARG for
 * null pointers). */
int scft_spline(int n, int end1, int end2, double slope1, double slope2, const double *x,
                const double *y, double *b, double *c, double *d, int *iflag);
/* seval (spline.c:213-278): S(u); *last is the segment hint, updated. */
double scft_spline_eval(int n, double u, const double *x, const double *y, const double *b,
                        const double *c, const double *d, int *last);
/* deriv (spline.c:281-347): S'(u). */
double scft_spline_deriv(int n, double u, const double *x, const double *b, const double *c,
                         const double *d, int *last);
/* sinteg (spline.c:351-433): the integral of S from x[0] to u. */
double scft_spline_integral(int n, double u, const double *x, const double *y, const double *b,
                            const double *c, const double *d, int *last);
/* Batched evaluation on the device (no reference counterpart): out[k] =
 * S(u[k]) (mode 0), S'(u[k]) (mode 1) or the integral to u[k] (mode 2); all
 * pointers are device memory; enqueued on `stream` (a cudaStream_t). */
int scft_spline_eval_device(int n, const double *x, const double *y, const double *b,
                            const double *c, const double *d, const double *u, double *out,
                            long long count, int mode, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SCFT_CAPI_H */
