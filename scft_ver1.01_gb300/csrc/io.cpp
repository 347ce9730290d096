// Drop-in file formats of the reference: ab.txt (init.cpp:81-94),
// phi_<i>.dat input (init_cuda.cu:435-456) and pha_<i>.dat output
// (cuda_scft.cu:233-243).  Unlike the reference, a missing or malformed file
// is reported as SCFT_ERR_IO instead of crashing on fscanf(NULL).
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "ctx.h"

extern "C" {

int scft_read_ab_txt(const char *path, scft_params *p, int *intag) {
  if (!path || !p) return SCFT_ERR_INVALID_ARG;
  FILE *fp = fopen(path, "r");
  if (!fp) return scft_fail(nullptr, SCFT_ERR_IO, std::string("cannot open ") + path);
  scft_params_default(p);
  int tag = 0, n = 0;
  n += fscanf(fp, "intag=%d\n", &tag);
  n += fscanf(fp, "xN=%lf\n", &p->hAB);
  n += fscanf(fp, "fa=%lf\n", &p->fA);
  n += fscanf(fp, "lx=%lf, ly=%lf, lz=%lf\n", &p->lx, &p->ly, &p->lz);
  n += fscanf(fp, "Nx=%d, Ny=%d, Nz=%d\n", &p->nx, &p->ny, &p->nz);
  n += fscanf(fp, "ds0=%lf\n", &p->ds0);
  n += fscanf(fp, "batch=%d\n", &p->batch);
  fclose(fp);
  if (n != 11) return scft_fail(nullptr, SCFT_ERR_IO, std::string("malformed ab.txt: ") + path);
  if (intag) *intag = tag;
  return SCFT_OK;
}

int scft_read_phi_dat(scft_ctx *ctx, const char *path, int inst) {
  if (!ctx || !path) return SCFT_ERR_INVALID_ARG;
  if (inst < 0 || inst >= ctx->batch) return scft_fail(ctx, SCFT_ERR_INVALID_ARG, "bad instance");
  FILE *fp = fopen(path, "r");
  if (!fp) return scft_fail(ctx, SCFT_ERR_IO, std::string("cannot open ") + path);
  char line[512];
  if (!fgets(line, sizeof line, fp) || !fgets(line, sizeof line, fp)) {
    fclose(fp);
    return scft_fail(ctx, SCFT_ERR_IO, std::string("missing header in ") + path);
  }
  const long long M = ctx->M;
  std::vector<double> a(M), b(M), c(M), d(M);
  for (long long i = 0; i < M; ++i) {
    if (fscanf(fp, "%lg %lg %lg %lg\n", &a[i], &b[i], &c[i], &d[i]) != 4) {
      fclose(fp);
      return scft_fail(ctx, SCFT_ERR_IO, std::string("short or malformed field file ") + path);
    }
  }
  fclose(fp);
  double *dst[4] = {ctx->pha, ctx->phb, ctx->wa, ctx->wb};
  ctx->and_count = 0;   // new fields: the Anderson history restarts
  std::vector<double> *src[4] = {&a, &b, &c, &d};
  cudaSetDevice(ctx->p.device);
  for (int k = 0; k < 4; ++k) {
    cudaError_t e = cudaMemcpy(dst[k] + (long long)inst * M, src[k]->data(), sizeof(double) * M,
                               cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return scft_fail(ctx, SCFT_ERR_CUDA, cudaGetErrorString(e));
  }
  return SCFT_OK;
}

int scft_write_pha_dat(scft_ctx *ctx, const char *path, int inst) {
  if (!ctx || !path) return SCFT_ERR_INVALID_ARG;
  if (inst < 0 || inst >= ctx->batch) return scft_fail(ctx, SCFT_ERR_INVALID_ARG, "bad instance");
  const long long M = ctx->M;
  std::vector<double> a(M), b(M), c(M), d(M);
  const double *src[4] = {ctx->pha, ctx->phb, ctx->wa, ctx->wb};
  std::vector<double> *dst[4] = {&a, &b, &c, &d};
  cudaSetDevice(ctx->p.device);
  cudaError_t e = cudaStreamSynchronize(ctx->st);
  if (e != cudaSuccess) return scft_fail(ctx, SCFT_ERR_CUDA, cudaGetErrorString(e));
  for (int k = 0; k < 4; ++k) {
    e = cudaMemcpy(dst[k]->data(), src[k] + (long long)inst * M, sizeof(double) * M,
                   cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return scft_fail(ctx, SCFT_ERR_CUDA, cudaGetErrorString(e));
  }
  FILE *dp = fopen(path, "w");
  if (!dp) return scft_fail(ctx, SCFT_ERR_IO, std::string("cannot write ") + path);
  const scft_params &p = ctx->p;
  fprintf(dp, "Nx=%d, Ny=%d, Nz=%d\n", p.nx, p.ny, p.nz);
  fprintf(dp, "dx=%g, dy=%g, dz=%g\n", p.lx / (double)p.nx, p.ly / (double)p.ny,
          p.lz / (double)p.nz);
  for (long long i = 0; i < M; ++i) fprintf(dp, "%g %g %g %g\n", a[i], b[i], c[i], d[i]);
  fclose(dp);
  return SCFT_OK;
}

}  // extern "C"
