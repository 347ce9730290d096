// The reference's C++ driver/struct API (include/compat/*.h) implemented on
// the C ABI, so the reference's driver (main.cpp:20-41) links against this
// library unchanged.  -GPU_N / -gpu<i> split the instances over devices as
// the reference does (init_cuda.cu:312): one context (shard) per listed
// device, each holding Num_SCFT / GPU_N instances, every call applied to all
// shards, no data moving between devices.  Errors print a message and leave
// the structs in a state finalize_cufft accepts; nothing calls exit() except
// init_scft on an unreadable ab.txt, where the reference itself would crash
// (init.cpp:81-86).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

#include <chrono>
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
// Refresh shard g's reference-layout mirror of propagator q (no-op without them).
void refresh_mirror(CUFFT_INFO *c, int g, int q) {
  if (!c->reference_layout) return;
  std::vector<double *> *mir[4] = {&c->qa_cu, &c->qcb_cu, &c->qb_cu, &c->qca_cu};
  report(c->shard[g], scft_copy_q_reference_layout(c->shard[g], q, (*mir[q])[g]),
         "reference layout");
}

// Make shard g's device current (each shard's calls run on its own device).
scft_ctx *use_shard(CUFFT_INFO *c, int g) {
  cudaSetDevice(c->shard[g]->p.device);
  return c->shard[g];
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

// init_cuda.cu:227-294 (device selection).  Peer access is not enabled: the
// shards never read each other's memory.
void init_cuda(GPU_INFO *gpu_info, int display) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess) ndev = 0;
  for (int i = 0; i < gpu_info->GPU_N && i < 64; ++i) {
    const int dev = gpu_info->whichGPUs[i];
    if (dev < 0 || dev >= ndev) continue;   // refused by initialize_cufft
    cudaGetDeviceProperties(&gpu_info->prop[i], dev);
    cudaSetDevice(dev);
    if (display == 1) printf("> GPU%d = \"%15s\"\n", i, gpu_info->prop[i].name);
  }
  if (gpu_info->GPU_N >= 1 && gpu_info->whichGPUs[0] >= 0 && gpu_info->whichGPUs[0] < ndev)
    cudaSetDevice(gpu_info->whichGPUs[0]);
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

  // the reference's split (init_cuda.cu:312): Num_SCFT / GPU_N per device
  const int n_gpu = gpu_info->GPU_N;
  int per = 0, not_run = 0;
  int st = scft_shard_plan(c->Num_SCFT, n_gpu, &per, &not_run);
  if (st != SCFT_OK) {
    report(nullptr, st, "initialize_cufft");
    return;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess) ndev = 0;
  for (int g = 0; g < n_gpu; ++g)
    if (gpu_info->whichGPUs[g] < 0 || gpu_info->whichGPUs[g] >= ndev) {
      fprintf(stderr, "initialize_cufft: -gpu%d=%d names no device (%d visible)\n", g,
              gpu_info->whichGPUs[g], ndev);
      return;
    }
  c->batch = per;
  if (not_run)
    printf("Instances %d to %d are not run: Num_SCFT %% GPU_N = %d (batch = Num_SCFT/GPU_N).\n",
           n_gpu * per + 1, c->Num_SCFT, not_run);
  scft_params p = c->opts;   // ab.txt's optional keys (defaults when absent)
  if (p.ds0 == 0.0) scft_params_default(&p);   // not parsed by init_scft: the defaults
  p.nx = Nx; p.ny = Ny; p.nz = Nz;
  p.lx = c->lx; p.ly = c->ly; p.lz = c->lz;
  p.hAB = c->hAB; p.fA = c->fA; p.ds0 = c->ds0;
  p.batch = c->batch;
  p.precision = c->precision;
  for (int g = 0; g < n_gpu; ++g) {
    p.device = gpu_info->whichGPUs[g];
    st = scft_create(&p, &c->shard[g]);
    if (st != SCFT_OK) {
      report(nullptr, st, "initialize_cufft");
      for (int k = 0; k < g; ++k) scft_destroy(c->shard[k]);
      for (int k = 0; k < n_gpu; ++k) c->shard[k] = nullptr;
      c->gb300 = nullptr;
      return;
    }
  }
  c->n_shard = n_gpu;
  c->gb300 = c->shard[0];
  printf("Wonderful We have successfully initialized GPU setting.\n");
  printf("Wonderful We have successfully initialized cufft setting.\n");
  if (c->metrics[0])
    for (int g = 0; g < n_gpu; ++g) scft_set_metrics_file(c->shard[g], c->metrics);
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
  gpu_info->stream = (cudaStream_t *)malloc(sizeof(cudaStream_t) * n_gpu);
  for (int g = 0; g < n_gpu; ++g) gpu_info->stream[g] = c->shard[g]->st;
  // initial fields (init_cuda.cu:435-456): global instance g*batch + i of
  // shard g reads phi_<g*batch+i+1>.dat
  if (c->intag == 1024) {
    for (int g = 0; g < n_gpu; ++g) {
      scft_ctx *ctx = use_shard(c, g);
      for (int i = 0; i < per; i++) {
        char name[64];
        snprintf(name, sizeof name, "phi_%d.dat", g * per + i + 1);
        st = scft_read_phi_dat(ctx, name, i);
        if (st != SCFT_OK) {
          printf("Configration file %s did not exist, please check it in your directory.\n",
                 name);
          report(ctx, st, "initialize_cufft");
        }
      }
      const long off = (long)g * per * M;
      scft_get_field(ctx, SCFT_FIELD_WA, c->wa + off);
      scft_get_field(ctx, SCFT_FIELD_WB, c->wb + off);
      scft_get_field(ctx, SCFT_FIELD_PHA, c->pha + off);
      scft_get_field(ctx, SCFT_FIELD_PHB, c->phb + off);
    }
  }
  printf("Wonderful We have successfully initialized CPU setting.\n");
  std::vector<double *> *mir[4] = {&c->qa_cu, &c->qcb_cu, &c->qb_cu, &c->qca_cu};
  for (std::vector<double *> *v : {&c->wa_cu, &c->wb_cu, &c->pha_cu, &c->phb_cu, &c->qa_cu,
                                   &c->qcb_cu, &c->qb_cu, &c->qca_cu, &c->qInt_cu, &c->wdz_cu,
                                   &c->ql, &c->ffl})
    v->assign(n_gpu, nullptr);
  for (int g = 0; g < n_gpu; ++g) {
    scft_ctx *ctx = c->shard[g];
    c->wa_cu[g] = ctx->wa;
    c->wb_cu[g] = ctx->wb;
    c->pha_cu[g] = ctx->pha;
    c->phb_cu[g] = ctx->phb;
    for (int q = 0; q < 4; ++q) (*mir[q])[g] = static_cast<double *>(ctx->q[q]);
    c->qInt_cu[g] = static_cast<double *>(ctx->qint);
    c->wdz_cu[g] = static_cast<double *>(ctx->W[0]);
    c->ql[g] = (double *)calloc(c->batch, sizeof(double));
    c->ffl[g] = (double *)calloc(c->batch, sizeof(double));
  }
  if (c->reference_layout) {
    // FP64 mirrors in the reference's g[b][r][s] layout (init_cuda.cu:522-526)
    std::vector<double *> m(4 * (size_t)n_gpu, nullptr);
    bool ok = true;
    for (int g = 0; g < n_gpu && ok; ++g) {
      scft_ctx *ctx = use_shard(c, g);
      for (int q = 0; q < 4 && ok; ++q)
        ok = cudaMalloc(&m[4 * g + q],
                        sizeof(double) * ctx->M * ctx->batch * (ctx->q_ns[q] + 1)) == cudaSuccess;
    }
    if (ok) {
      for (int g = 0; g < n_gpu; ++g)
        for (int q = 0; q < 4; ++q) (*mir[q])[g] = m[4 * g + q];
    } else {
      cudaGetLastError();
      for (int g = 0; g < n_gpu; ++g) {
        use_shard(c, g);
        for (int q = 0; q < 4; ++q) cudaFree(m[4 * g + q]);
      }
      fprintf(stderr, "initialize_cufft: cannot allocate the reference-layout propagators; "
                      "keeping the contour-outer ones\n");
      c->reference_layout = 0;
    }
  }
  use_shard(c, 0);
  printf("Wonderful We have successfully initialized all the data.\n");
}

// cuda_scft.cu:14-59: every shard's instances (data[g] is shard g's array)
void average_value(std::vector<double *> data, GPU_INFO *gpu_info, CUFFT_INFO *c) {
  (void)gpu_info;
  if (!c->gb300 || data.empty()) return;
  const int f = field_of(c, data[0]);
  if (f < 0) {
    fprintf(stderr, "average_value: pointer is not wa_cu or wb_cu\n");
    return;
  }
  for (int g = 0; g < c->n_shard; ++g)
    report(c->shard[g], scft_average_value(use_shard(c, g), f), "average_value");
  for (int g = 0; g < c->n_shard; ++g) scft_synchronize(use_shard(c, g));
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
  for (int k = 0; k < c->n_shard; ++k)
    report(c->shard[k], scft_sov_dif_fft(use_shard(c, k), q, f, ns, sign), "sovDifFft");
  for (int k = 0; k < c->n_shard; ++k) {
    scft_synchronize(use_shard(c, k));
    refresh_mirror(c, k, q);
  }
}

// cuda_scft.cu:61-138: queued on every shard before any is waited for
void getConc(GPU_INFO *gpu_info, CUFFT_INFO *c) {
  (void)gpu_info;
  if (!c->gb300) return;
  for (int g = 0; g < c->n_shard; ++g)
    report(c->shard[g], scft_get_conc(use_shard(c, g)), "getConc");
  for (int g = 0; g < c->n_shard; ++g) {
    scft_ctx *ctx = use_shard(c, g);
    for (int q = 0; q < 4; ++q) refresh_mirror(c, g, q);
    if (scft_get_Q(ctx, c->ql[g]) == SCFT_OK)
      for (int i = 0; i < c->batch; ++i) c->ffl[g][i] = c->ds0 / c->ql[g][i];
  }
}

// cuda_scft.cu:140-269: prints the progress lines and writes pha_<i>.dat in
// the working directory, as the reference does, over every shard.
double Free(GPU_INFO *gpu_info, CUFFT_INFO *c) {
  (void)gpu_info;
  if (!c->gb300) return 0;
  report(c->gb300, scft_free_shards(c->shard, c->n_shard, c->MaxIT, c->AverIt, "."), "Free");
  for (int g = 0; g < c->n_shard; ++g) scft_get_Q(use_shard(c, g), c->ql[g]);
  use_shard(c, 0);
  return 0;
}

// cuda_scft.cu:382-432.  The reference brackets Free with events on the
// current device's default stream; Free synchronises every device before it
// returns, so the host clock measures the same interval on any number of
// shards.
void fft_test(GPU_INFO *gpu_info, CUFFT_INFO *c) {
  if (!c->gb300) {
    printf("fft_test did not successfully detect run time\n");
    return;
  }
  const auto t0 = std::chrono::steady_clock::now();
  Free(gpu_info, c);
  const double msec =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  printf("time=%0.10f\n", msec);
}

// init_cuda.cu:551-628
void finalize_cufft(GPU_INFO *gpu_info, CUFFT_INFO *c) {
  std::vector<double *> *mir[4] = {&c->qa_cu, &c->qcb_cu, &c->qb_cu, &c->qca_cu};
  for (int g = 0; g < c->n_shard; ++g) {
    if (!c->shard[g]) continue;
    use_shard(c, g);
    if (c->reference_layout)
      for (auto *m : mir)
        if ((int)m->size() > g) cudaFree((*m)[g]);
    scft_destroy(c->shard[g]);
    c->shard[g] = nullptr;
  }
  c->n_shard = 0;
  c->gb300 = nullptr;
  free(c->wa); free(c->wb); free(c->pha); free(c->phb);
  free(c->kx); free(c->ky); free(c->kz); free(c->kxyzdz);
  for (double *q : c->ql) free(q);
  for (double *f : c->ffl) free(f);
  c->ql.clear();
  c->ffl.clear();
  free(gpu_info->stream);
  free(gpu_info->whichGPUs);
  gpu_info->stream = nullptr;
  gpu_info->whichGPUs = nullptr;
  printf("Wonderful We have successfully evaculate all the memery on GPU and CPU \n");
}
