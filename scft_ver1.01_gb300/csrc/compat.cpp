// The reference's C++ driver/struct API (include/compat/*.h) implemented on
// the C ABI, so the reference's driver (main.cpp:20-41) links against this
// library unchanged.  One GPU: the reference's GPU_N split of `batch`
// (init_cuda.cu:312) collapses onto the first listed device.  Errors print a
// message and leave the structs in a state finalize_cufft accepts; nothing
// calls exit() except init_scft on an unreadable ab.txt, where the reference
// itself would crash (init.cpp:81-86).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

#include <string>

#include "compat/cuda_scft.h"
#include "compat/init.h"
#include "compat/init_cuda.h"
#include "ctx.h"

namespace {

// "-name=value" / "--name=value" lookup (the CUDA-samples helpers the
// reference uses, init.cpp:14-37).
const char *flag_value(int argc, char **argv, const char *name) {
  const size_t n = strlen(name);
  for (int i = 1; i < argc; ++i) {
    const char *a = argv[i];
    while (*a == '-') ++a;
    if (strncmp(a, name, n) == 0 && a[n] == '=') return a + n + 1;
  }
  return nullptr;
}
int flag_int(int argc, char **argv, const char *name) {
  const char *v = flag_value(argc, argv, name);
  return v ? atoi(v) : 0;
}

void report(scft_ctx *ctx, int st, const char *where) {
  if (st != SCFT_OK)
    fprintf(stderr, "%s: %s (%s)\n", where, scft_strerror(st), scft_last_error(ctx));
}

int field_of(CUFFT_INFO *c, double *p) {
  if (!c->wa_cu.empty() && p == c->wa_cu[0]) return SCFT_FIELD_WA;
  if (!c->wb_cu.empty() && p == c->wb_cu[0]) return SCFT_FIELD_WB;
  return -1;
}
// Refresh the reference-layout mirror of propagator q (no-op without them).
void refresh_mirror(CUFFT_INFO *c, int q) {
  if (!c->reference_layout) return;
  std::vector<double *> *mir[4] = {&c->qa_cu, &c->qcb_cu, &c->qb_cu, &c->qca_cu};
  report(c->gb300, scft_copy_q_reference_layout(c->gb300, q, (*mir[q])[0]), "reference layout");
}

int prop_of(CUFFT_INFO *c, double *p) {
  if (!c->qa_cu.empty() && p == c->qa_cu[0]) return SCFT_Q_A;
  if (!c->qcb_cu.empty() && p == c->qcb_cu[0]) return SCFT_Q_CB;
  if (!c->qb_cu.empty() && p == c->qb_cu[0]) return SCFT_Q_B;
  if (!c->qca_cu.empty() && p == c->qca_cu[0]) return SCFT_Q_CA;
  return -1;
}

int largest_divisor_1024(long n) {
  int best = 1;
  for (int d = 1; d <= 1024 && d <= n; ++d)
    if (n % d == 0) best = d;
  return best;
}

}  // namespace

// init.cpp:8-132
int init_scft(CUFFT_INFO *cufft_info, GPU_INFO *gpu_info, int argc, char **argv) {
  memset(gpu_info, 0, sizeof(*gpu_info));
  // the layout choice comes from the driver's own compilation of struct.h
  // (its default member initializer), so it survives the reset
  const int layout = cufft_info->reference_layout == 1 ? 1 : 0;
  new (cufft_info) CUFFT_INFO();
  cufft_info->reference_layout = layout;
  gpu_info->kernal_type = -1;
  const char *type = flag_value(argc, argv, "kernal");
  cufft_info->MaxIT = flag_int(argc, argv, "step");
  gpu_info->GPU_N = flag_int(argc, argv, "GPU_N");
  if (gpu_info->GPU_N == 0) gpu_info->GPU_N = 1;
  gpu_info->whichGPUs = (int *)malloc(sizeof(int) * gpu_info->GPU_N);
  for (int i = 0; i < gpu_info->GPU_N; i++) {
    char name[20];
    snprintf(name, sizeof name, "gpu%d", i);
    gpu_info->whichGPUs[i] = flag_int(argc, argv, name);
  }
  cufft_info->AverIt = 10;
  if (cufft_info->MaxIT < 1) {
    printf("Maximal iterative step did not set, defalt set as 100.\n");
    cufft_info->MaxIT = 100;
    printf("It could as well be set by adding flag -step=Num. \n");
  }
  const char *prec = flag_value(argc, argv, "precision");
  cufft_info->precision = !prec                      ? SCFT_PREC_FP64
                          : !strcasecmp(prec, "fp32") ? SCFT_PREC_FP32
                          : !strcasecmp(prec, "df")   ? SCFT_PREC_DF
                                                      : SCFT_PREC_FP64;
  const char *metrics = flag_value(argc, argv, "metrics");
  snprintf(cufft_info->metrics, sizeof cufft_info->metrics, "%s", metrics ? metrics : "");
  if (type) {
    if (!strcasecmp(type, "GPU")) gpu_info->kernal_type = 1;
    else if (!strcasecmp(type, "CPU")) gpu_info->kernal_type = 2;
    else gpu_info->kernal_type = -1;
  } else {
    gpu_info->kernal_type = 1;
  }
  if (gpu_info->kernal_type == 1) {
    printf("In this programm, we use GPU.\n");
    scft_params p;
    int intag = 0;
    if (scft_read_ab_txt("ab.txt", &p, &intag) != SCFT_OK) {
      printf("Configration file ab.txt did not exist, please check it in your directory.\n");
      fprintf(stderr, "%s\n", scft_last_error(nullptr));
      exit(1);
    }
    cufft_info->intag = intag;
    cufft_info->opts = p;
    if (!prec) cufft_info->precision = p.precision;   // the -precision flag wins over ab.txt
    cufft_info->hAB = p.hAB;
    cufft_info->fA = p.fA;
    cufft_info->lx = p.lx; cufft_info->ly = p.ly; cufft_info->lz = p.lz;
    cufft_info->Nx = p.nx; cufft_info->Ny = p.ny; cufft_info->Nz = p.nz;
    cufft_info->ds0 = p.ds0;
    cufft_info->Num_SCFT = p.batch;
    cufft_info->batch = p.batch;
    init_cuda(gpu_info, 0);
    initialize_cufft(gpu_info, cufft_info);
  } else if (gpu_info->kernal_type == 2) {
    printf("In this programm, we use CPU.\n");
  } else {
    printf("Set kernal type by adding flag -kernal=GPU/CPU, but CPU now is not aviliable\n");
  }
  return 0;
}

// init_cuda.cu:227-294 (device selection; peer access is not needed)
void init_cuda(GPU_INFO *gpu_info, int display) {
  if (gpu_info->GPU_N > 1)
    printf("GB300 build: %d GPUs requested; all instances run on GPU %d.\n", gpu_info->GPU_N,
           gpu_info->whichGPUs[0]);
  cudaGetDeviceProperties(&gpu_info->prop[0], gpu_info->whichGPUs[0]);
  cudaSetDevice(gpu_info->whichGPUs[0]);
  if (display == 1)
    printf("> GPU%d = \"%15s\"\n", gpu_info->whichGPUs[0], gpu_info->prop[0].name);
}

// init_cuda.cu:296-546
void initialize_cufft(GPU_INFO *gpu_info, CUFFT_INFO *c) {
  const int Nx = c->Nx, Ny = c->Ny, Nz = c->Nz;
  c->NxNyNz = (long)Nx * Ny * Nz;
  c->Nxh1 = Nx / 2 + 1;
  c->Nxh1NyNz = (long)c->Nxh1 * Ny * Nz;
  c->batch = c->Num_SCFT;   // one GPU holds every instance
  gpu_info->thread = largest_divisor_1024(c->NxNyNz);
  gpu_info->thread_sur = largest_divisor_1024(c->Nxh1NyNz);
  c->ds2 = c->ds0 / 2;
  c->dfB = 1 - c->fA;
  c->fB = c->dfB;
  c->NsA = (int)(c->fA / c->ds0 + 1.0e-8);
  c->dNsB = (int)(c->dfB / c->ds0 + 1.0e-8);
  c->NsB = c->dNsB;
  c->ns = c->NsA + c->dNsB;
  c->dx = c->lx / (double)Nx;
  c->dy = c->ly / (double)Ny;
  c->dz = c->lz / (double)Nz;

  scft_params p = c->opts;   // ab.txt's optional keys (defaults when absent)
  if (p.ds0 == 0.0) scft_params_default(&p);   // not parsed by init_scft: the defaults
  p.nx = Nx; p.ny = Ny; p.nz = Nz;
  p.lx = c->lx; p.ly = c->ly; p.lz = c->lz;
  p.hAB = c->hAB; p.fA = c->fA; p.ds0 = c->ds0;
  p.batch = c->batch;
  p.precision = c->precision;
  p.device = gpu_info->whichGPUs ? gpu_info->whichGPUs[0] : 0;
  int st = scft_create(&p, &c->gb300);
  if (st != SCFT_OK) {
    report(nullptr, st, "initialize_cufft");
    c->gb300 = nullptr;
    return;
  }
  printf("Wonderful We have successfully initialized GPU setting.\n");
  printf("Wonderful We have successfully initialized cufft setting.\n");
  scft_ctx *ctx = c->gb300;
  if (c->metrics[0]) scft_set_metrics_file(ctx, c->metrics);
  const long M = c->NxNyNz;
  // host arrays and wave-number tables (init_cuda.cu:380-428)
  c->wa = (double *)calloc(M * c->Num_SCFT, sizeof(double));
  c->wb = (double *)calloc(M * c->Num_SCFT, sizeof(double));
  c->pha = (double *)calloc(M * c->Num_SCFT, sizeof(double));
  c->phb = (double *)calloc(M * c->Num_SCFT, sizeof(double));
  c->kx = (double *)malloc(sizeof(double) * Nx);
  c->ky = (double *)malloc(sizeof(double) * Ny);
  c->kz = (double *)malloc(sizeof(double) * Nz);
  double *ks[3] = {c->kx, c->ky, c->kz};
  const int ns3[3] = {Nx, Ny, Nz};
  const double ds3[3] = {c->dx, c->dy, c->dz};
  for (int a = 0; a < 3; ++a) {
    const int n = ns3[a];
    for (int i = 0; i <= n / 2 - 1; i++) ks[a][i] = 2 * Pi * i * 1.0 / n / ds3[a];
    for (int i = n / 2; i < n; i++) ks[a][i] = 2 * Pi * (i - n) * 1.0 / ds3[a] / n;
    for (int i = 0; i < n; i++) ks[a][i] *= ks[a][i];
  }
  c->kxyzdz = (double *)malloc(sizeof(double) * M);
  for (int k = 0; k < Nz; k++)
    for (int j = 0; j < Ny; j++)
      for (int i = 0; i < Nx; i++)
        c->kxyzdz[(long)(k * Ny + j) * Nx + i] = exp(-c->ds0 * (c->kx[i] + c->ky[j] + c->kz[k]));
  gpu_info->stream = (cudaStream_t *)malloc(sizeof(cudaStream_t));
  gpu_info->stream[0] = ctx->st;
  // initial fields (init_cuda.cu:435-456)
  if (c->intag == 1024) {
    for (int i = 0; i < c->Num_SCFT; i++) {
      char name[64];
      snprintf(name, sizeof name, "phi_%d.dat", i + 1);
      st = scft_read_phi_dat(ctx, name, i);
      if (st != SCFT_OK) {
        printf("Configration file %s did not exist, please check it in your directory.\n", name);
        report(ctx, st, "initialize_cufft");
      }
    }
    scft_get_field(ctx, SCFT_FIELD_WA, c->wa);
    scft_get_field(ctx, SCFT_FIELD_WB, c->wb);
    scft_get_field(ctx, SCFT_FIELD_PHA, c->pha);
    scft_get_field(ctx, SCFT_FIELD_PHB, c->phb);
  }
  printf("Wonderful We have successfully initialized CPU setting.\n");
  c->wa_cu.assign(1, ctx->wa);
  c->wb_cu.assign(1, ctx->wb);
  c->pha_cu.assign(1, ctx->pha);
  c->phb_cu.assign(1, ctx->phb);
  c->qa_cu.assign(1, static_cast<double *>(ctx->q[SCFT_Q_A]));
  c->qcb_cu.assign(1, static_cast<double *>(ctx->q[SCFT_Q_CB]));
  c->qb_cu.assign(1, static_cast<double *>(ctx->q[SCFT_Q_B]));
  c->qca_cu.assign(1, static_cast<double *>(ctx->q[SCFT_Q_CA]));
  if (c->reference_layout) {
    // FP64 mirrors in the reference's g[b][r][s] layout (init_cuda.cu:522-526)
    std::vector<double *> *mir[4] = {&c->qa_cu, &c->qcb_cu, &c->qb_cu, &c->qca_cu};
    double *m[4] = {nullptr, nullptr, nullptr, nullptr};
    bool ok = true;
    for (int q = 0; q < 4 && ok; ++q)
      ok = cudaMalloc(&m[q], sizeof(double) * ctx->M * ctx->batch * (ctx->q_ns[q] + 1)) ==
           cudaSuccess;
    if (ok) {
      for (int q = 0; q < 4; ++q) mir[q]->assign(1, m[q]);
    } else {
      cudaGetLastError();
      for (double *p : m) cudaFree(p);
      fprintf(stderr, "initialize_cufft: cannot allocate the reference-layout propagators; "
                      "keeping the contour-outer ones\n");
      c->reference_layout = 0;
    }
  }
  c->qInt_cu.assign(1, static_cast<double *>(ctx->qint));
  c->wdz_cu.assign(1, static_cast<double *>(ctx->W[0]));
  c->ql.assign(1, (double *)calloc(c->batch, sizeof(double)));
  c->ffl.assign(1, (double *)calloc(c->batch, sizeof(double)));
  printf("Wonderful We have successfully initialized all the data.\n");
}

// cuda_scft.cu:14-59
void average_value(std::vector<double *> data, GPU_INFO *gpu_info, CUFFT_INFO *c) {
  (void)gpu_info;
  if (!c->gb300 || data.empty()) return;
  const int f = field_of(c, data[0]);
  if (f < 0) {
    fprintf(stderr, "average_value: pointer is not wa_cu or wb_cu\n");
    return;
  }
  report(c->gb300, scft_average_value(c->gb300, f), "average_value");
  scft_synchronize(c->gb300);
}

// cuda_scft.cu:435-563
void sovDifFft(GPU_INFO *gpu_info, CUFFT_INFO *c, std::vector<double *> g,
               std::vector<double *> w, int ns, int sign) {
  (void)gpu_info;
  if (!c->gb300 || g.empty() || w.empty()) return;
  const int q = prop_of(c, g[0]), f = field_of(c, w[0]);
  if (q < 0 || f < 0) {
    fprintf(stderr, "sovDifFft: unknown propagator or field pointer\n");
    return;
  }
  report(c->gb300, scft_sov_dif_fft(c->gb300, q, f, ns, sign), "sovDifFft");
  scft_synchronize(c->gb300);
  refresh_mirror(c, q);
}

// cuda_scft.cu:61-138
void getConc(GPU_INFO *gpu_info, CUFFT_INFO *c) {
  (void)gpu_info;
  if (!c->gb300) return;
  report(c->gb300, scft_get_conc(c->gb300), "getConc");
  for (int q = 0; q < 4; ++q) refresh_mirror(c, q);
  if (scft_get_Q(c->gb300, c->ql[0]) == SCFT_OK)
    for (int i = 0; i < c->batch; ++i) c->ffl[0][i] = c->ds0 / c->ql[0][i];
}

// cuda_scft.cu:140-269: prints the progress lines and writes pha_<i>.dat in
// the working directory, as the reference does.
double Free(GPU_INFO *gpu_info, CUFFT_INFO *c) {
  (void)gpu_info;
  if (!c->gb300) return 0;
  report(c->gb300, scft_free(c->gb300, c->MaxIT, c->AverIt, "."), "Free");
  scft_get_Q(c->gb300, c->ql[0]);
  return 0;
}

// cuda_scft.cu:382-432
void fft_test(GPU_INFO *gpu_info, CUFFT_INFO *c) {
  if (!c->gb300) {
    printf("fft_test did not successfully detect run time\n");
    return;
  }
  cudaEvent_t start, stop;
  float msec = 0.f;
  cudaEventCreate(&start);
  cudaEventCreate(&stop);
  cudaEventRecord(start, c->gb300->st);
  Free(gpu_info, c);
  cudaEventRecord(stop, c->gb300->st);
  cudaEventSynchronize(stop);
  if (cudaEventElapsedTime(&msec, start, stop) != cudaSuccess)
    printf("fft_test did not successfully detect run time\n");
  printf("time=%0.10f\n", msec);
  cudaEventDestroy(start);
  cudaEventDestroy(stop);
}

// init_cuda.cu:551-628
void finalize_cufft(GPU_INFO *gpu_info, CUFFT_INFO *c) {
  if (c->reference_layout && c->gb300) {
    std::vector<double *> *mir[4] = {&c->qa_cu, &c->qcb_cu, &c->qb_cu, &c->qca_cu};
    for (auto *m : mir)
      if (!m->empty()) cudaFree((*m)[0]);
  }
  if (c->gb300) scft_destroy(c->gb300);
  c->gb300 = nullptr;
  free(c->wa); free(c->wb); free(c->pha); free(c->phb);
  free(c->kx); free(c->ky); free(c->kz); free(c->kxyzdz);
  if (!c->ql.empty()) free(c->ql[0]);
  if (!c->ffl.empty()) free(c->ffl[0]);
  free(gpu_info->stream);
  free(gpu_info->whichGPUs);
  gpu_info->stream = nullptr;
  gpu_info->whichGPUs = nullptr;
  printf("Wonderful We have successfully evaculate all the memery on GPU and CPU \n");
}
