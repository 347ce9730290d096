/*
 * struct.h -- the reference's C++ struct API (GPU_INFO / CUFFT_INFO,
 * struct.h:19-125 of ren5885a/SCFT_Ver1.01) re-declared for the GB300 build,
 * so a driver written against the reference compiles unchanged.  Field names
 * and meanings are kept; the implementation behind them is the C ABI of
 * ../scft_capi.h.  -GPU_N / -gpu<i> split the instances over devices as the
 * reference does (batch = Num_SCFT / GPU_N per device, init_cuda.cu:312), one
 * context per device, with no data moving between them.  Differences a
 * caller can observe:
 *   - the *_cu vectors hold one device pointer per shard (index gpu_index),
 *     as the reference's do;
 *   - wa_cu/wb_cu/pha_cu/phb_cu are FP64 [batch][Nz][Ny][Nx] device arrays;
 *   - qa_cu/qb_cu/qca_cu/qcb_cu point at contour-outer propagator storage
 *     ([batch][s][Nz][Ny][Nx] in the propagation precision: FP64, FP32, or
 *     double-float pairs {float hi, lo}), not the reference's s-fastest
 *     g[b][r][s] -- unless the driver is compiled with
 *     -DSCFT_COMPAT_FP64_LAYOUT: then they point at FP64 mirrors in the
 *     reference's layout, refreshed by getConc and sovDifFft;
 *   - ql/ffl hold host arrays (batch doubles), refreshed by getConc;
 *   - plan_forward/plan_backward/device_in/device_out/kxyzdz_cu are unused
 *     (the FFTs are the library's own kernels).
 */
#ifndef SCFT_GB300_COMPAT_STRUCT_H
#define SCFT_GB300_COMPAT_STRUCT_H

#include <cuda_runtime.h>
#include <cufft.h>

#include <vector>

#include "../scft_capi.h"

#define Pi 3.1415926535

#ifdef SCFT_COMPAT_FP64_LAYOUT
#define SCFT_COMPAT_REFERENCE_LAYOUT 1
#else
#define SCFT_COMPAT_REFERENCE_LAYOUT 0
#endif

typedef struct {
  int kernal_type;   /* 1 GPU, 2 CPU (not available), -1 unset */
  int GPU_N;
  int *whichGPUs;
  cudaStream_t *stream;
  int thread;        /* largest divisor of Nx*Ny*Nz <= 1024 (informational) */
  int thread_sur;
  cudaDeviceProp prop[64];
} GPU_INFO;

typedef struct {
  int batch;         /* instances per GPU (all of them: one GPU) */
  int Num_SCFT;
  int intag;
  double hAB;
  double fA;
  double fB;
  int MaxIT;
  int AverIt;
  int Nx, Ny, Nz, Nxh1;
  long NxNyNz;
  long Nxh1NyNz;
  int NsA, NsB, ns, dNsB;
  double dfB;
  double lx, ly, lz;
  double dx, dy, dz;
  double ds0, ds2;
  cufftHandle *plan_forward;
  cufftHandle *plan_backward;
  std::vector<double *> device_in;
  std::vector<cufftDoubleComplex *> device_out;
  double Sm1, Sm2;
  double *kx, *kz, *ky;
  double *wa, *wb, *wc;
  double *pha, *phb, *phc;
  double **kxyzdz_cu;
  double *kxyzdz;
  std::vector<double *> ql;
  std::vector<double *> ffl;
  std::vector<double *> pha_cu;
  std::vector<double *> phb_cu;
  std::vector<double *> wa_cu;
  std::vector<double *> wb_cu;
  std::vector<double *> qInt_cu;
  std::vector<double *> wdz_cu;
  std::vector<double *> qa_cu;
  std::vector<double *> qb_cu;
  std::vector<double *> qca_cu;
  std::vector<double *> qcb_cu;
  /* GB300 build: the context behind the fields above */
  scft_ctx *gb300;
  int precision;     /* SCFT_PREC_FP64 (default), SCFT_PREC_FP32 or SCFT_PREC_DF */
  /* 1: qa_cu/qb_cu/qca_cu/qcb_cu are FP64 mirrors in the reference's
   * g[b][r][s] layout (set by -DSCFT_COMPAT_FP64_LAYOUT in the driver) */
  int reference_layout = SCFT_COMPAT_REFERENCE_LAYOUT;
  /* ab.txt as parsed by scft_read_ab_txt, with its optional keys (mixing,
   * Anderson history/lambda/start, wopt, wcmp, precision, Ns) */
  scft_params opts = {};
  /* -metrics=<path>: JSON-lines progress reports (scft_set_metrics_file) */
  char metrics[256] = {};
  /* the contexts of the GPU_N split, one per listed device (gb300 == shard[0]) */
  scft_ctx *shard[SCFT_MAX_SHARDS] = {};
  int n_shard = 0;
} CUFFT_INFO;

#endif
