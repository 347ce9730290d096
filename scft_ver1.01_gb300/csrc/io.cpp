// Drop-in file formats of the reference: ab.txt (init.cpp:81-94),
// phi_<i>.dat input (init_cuda.cu:435-456), pha_<i>.dat output
// (cuda_scft.cu:233-243) and the VTK converter's output (vtk.c).  Unlike the reference, a missing or malformed file
// is reported as SCFT_ERR_IO instead of crashing on fscanf(NULL).
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
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
  if (n != 11) {
    fclose(fp);
    return scft_fail(nullptr, SCFT_ERR_IO, std::string("malformed ab.txt: ") + path);
  }
  // optional key=value lines after the reference's seven
  char line[256];
  while (fgets(line, sizeof line, fp)) {
    std::string l(line);
    while (!l.empty() && (l.back() == '\n' || l.back() == '\r' || l.back() == ' ')) l.pop_back();
    if (l.empty() || l[0] == '#') continue;   // blank lines and comments
    const size_t eq = l.find('=');
    std::string err;
    if (eq == std::string::npos) {
      err = "not a key=value line";
    } else {
      const std::string key = l.substr(0, eq), val = l.substr(eq + 1);
      char *end = nullptr;
      const double x = strtod(val.c_str(), &end);
      const bool num = end && end != val.c_str() && *end == '\0';
      if (key == "mixing") {
        if (val == "simple") p->mixing = SCFT_MIX_SIMPLE;
        else if (val == "anderson") p->mixing = SCFT_MIX_ANDERSON;
        else err = "mixing must be simple or anderson";
      } else if (key == "precision") {
        if (val == "fp32") p->precision = SCFT_PREC_FP32;
        else if (val == "fp64") p->precision = SCFT_PREC_FP64;
        else if (val == "df") p->precision = SCFT_PREC_DF;
        else err = "precision must be fp32, fp64 or df";
      } else if (!num) {
        err = "not a number";
      } else if (key == "history") {
        p->anderson_history = (int)x;
      } else if (key == "lambda") {
        p->anderson_lambda = x;
      } else if (key == "start") {
        p->anderson_start = x;
      } else if (key == "wopt") {
        p->wopt = x;
      } else if (key == "wcmp") {
        p->wcmp = x;
      } else if (key == "Ns") {
        if (x >= 1) p->ds0 = 1.0 / x;
        else err = "Ns must be >= 1";
      } else {
        err = "unknown key";
      }
    }
    if (!err.empty()) {
      fclose(fp);
      return scft_fail(nullptr, SCFT_ERR_IO,
                       std::string(path) + ": " + err + " in line '" + l + "'");
    }
  }
  fclose(fp);
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

namespace {

// The converter's output (vtk.c:54-76): a STRUCTURED_POINTS header with the
// spacing as read, then phiA - phiB as "%7.4lf " per point, x fastest, one
// text row per (z, y).  `diff` holds nx*ny*nz values in that order.
int write_vtk_file(const char *path, const char *source, int nx, int ny, int nz, double dx,
                   double dy, double dz, const std::vector<double> &diff) {
  FILE *fp = fopen(path, "w");
  if (!fp) return SCFT_ERR_IO;
  fprintf(fp, "# vtk DataFile Version 3.0\n");
  fprintf(fp, "# comment: converted from file %s\n", source);
  fprintf(fp, "ASCII\n");
  fprintf(fp, "DATASET STRUCTURED_POINTS\n");
  fprintf(fp, "DIMENSIONS %d %d %d\n", nx, ny, nz);
  fprintf(fp, "ORIGIN 0.000000 0.000000 0.000000\n");
  fprintf(fp, "SPACING %.6f %.6f %.6f\n\n", dx, dy, dz);
  fprintf(fp, "POINT_DATA %lld\n", (long long)nx * ny * nz);
  fprintf(fp, "SCALARS scalars float\n");
  fprintf(fp, "LOOKUP_TABLE default\n\n");
  // one row buffered at a time: a 128^3 field is 16K rows of 8*nx bytes
  std::string row;
  char cell[64];
  long long i = 0;
  for (long long r = 0; r < (long long)ny * nz; ++r) {
    row.clear();
    for (int x = 0; x < nx; ++x, ++i) {
      snprintf(cell, sizeof cell, "%7.4f ", diff[i]);
      row += cell;
    }
    row += '\n';
    fwrite(row.data(), 1, row.size(), fp);
  }
  return fclose(fp) == 0 ? SCFT_OK : SCFT_ERR_IO;
}

// A value as it survives the pha file's "%g" text (cuda_scft.cu:238).
double through_g(double v) {
  char t[64];
  snprintf(t, sizeof t, "%g", v);
  return strtod(t, nullptr);
}

}  // namespace

extern "C" {

int scft_convert_pha_to_vtk(const char *pha_path, const char *vtk_path) {
  const char *in = pha_path ? pha_path : "pha.dat";     // vtk.c:17-18 defaults
  const char *out = vtk_path ? vtk_path : "out.vtk";
  FILE *fp = fopen(in, "r");
  if (!fp) return scft_fail(nullptr, SCFT_ERR_IO, std::string("cannot open ") + in);
  int nx = 0, ny = 0, nz = 0;
  double dx = 0, dy = 0, dz = 0;
  int n = fscanf(fp, "Nx=%d, Ny=%d, Nz=%d\n", &nx, &ny, &nz);
  n += fscanf(fp, "dx=%lf, dy=%lf, dz=%lf\n", &dx, &dy, &dz);
  if (n != 6 || nx <= 0 || ny <= 0 || nz <= 0) {
    fclose(fp);
    return scft_fail(nullptr, SCFT_ERR_IO, std::string("malformed header in ") + in);
  }
  const long long M = (long long)nx * ny * nz;
  std::vector<double> diff(M);
  for (long long i = 0; i < M; ++i) {
    double a, b, c, d;
    if (fscanf(fp, "%lf %lf %lf %lf\n", &a, &b, &c, &d) != 4) {
      fclose(fp);
      return scft_fail(nullptr, SCFT_ERR_IO, std::string("short or malformed field file ") + in);
    }
    diff[i] = a - b;
  }
  fclose(fp);
  if (write_vtk_file(out, in, nx, ny, nz, dx, dy, dz, diff) != SCFT_OK)
    return scft_fail(nullptr, SCFT_ERR_IO, std::string("cannot write ") + out);
  return SCFT_OK;
}

int scft_write_vtk(scft_ctx *ctx, const char *path, int inst, const char *source) {
  if (!ctx || !path) return SCFT_ERR_INVALID_ARG;
  if (inst < 0 || inst >= ctx->batch) return scft_fail(ctx, SCFT_ERR_INVALID_ARG, "bad instance");
  const long long M = ctx->M;
  std::vector<double> a(M), b(M);
  cudaSetDevice(ctx->p.device);
  cudaError_t e = cudaStreamSynchronize(ctx->st);
  if (e == cudaSuccess)
    e = cudaMemcpy(a.data(), ctx->pha + (long long)inst * M, sizeof(double) * M,
                   cudaMemcpyDeviceToHost);
  if (e == cudaSuccess)
    e = cudaMemcpy(b.data(), ctx->phb + (long long)inst * M, sizeof(double) * M,
                   cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return scft_fail(ctx, SCFT_ERR_CUDA, cudaGetErrorString(e));
  // the same values the pha file -> converter route gives: phiA and phiB as
  // their "%g" text, the spacing as "%g" text
  for (long long i = 0; i < M; ++i) a[i] = through_g(a[i]) - through_g(b[i]);
  const scft_params &p = ctx->p;
  if (write_vtk_file(path, source ? source : "pha.dat", p.nx, p.ny, p.nz,
                     through_g(p.lx / (double)p.nx), through_g(p.ly / (double)p.ny),
                     through_g(p.lz / (double)p.nz), a) != SCFT_OK)
    return scft_fail(ctx, SCFT_ERR_IO, std::string("cannot write ") + path);
  return SCFT_OK;
}

}  // extern "C"

// ---- binary FP64 checkpoint (no reference counterpart) -------------------
//
// Layout (native byte order; both machines this builds for are little-endian):
//   char[8] "SCFTCKP2", int32 version (2),
//   int32 nx, ny, nz, batch, precision, mixing, anderson_history, has_history,
//   double lx, ly, lz, hAB, fA, ds0, int64 and_count, double anderson_lambda,
//   double wa, wb, phiA, phiB   [batch][M] each,
//   double residual             [batch][4]   (norms and means of the last update)
//   with has_history: int32 m1, then m1 rings of u = w + anderson_lambda d and
//   m1 rings of d ([batch][2][M] double-float pairs each: float hi, float lo,
//   the device ring's bytes) and the Gram matrix [batch][m1][m1] (double).
namespace {

struct CkptHeader {
  char magic[8];
  int32_t version, nx, ny, nz, batch, precision, mixing, history, has_history;
  double lx, ly, lz, hAB, fA, ds0;
  int64_t and_count;
  double anderson_lambda;
};

// device <-> file through a bounded host buffer, n 8-byte words copied as
// bytes (doubles, or double-float pairs)
int dev_to_file(scft_ctx *ctx, FILE *fp, const void *dev, long long n) {
  const long long chunk = 1LL << 23;   // 64 MB
  std::vector<uint64_t> buf((size_t)(n < chunk ? n : chunk));
  const uint64_t *src = static_cast<const uint64_t *>(dev);
  for (long long o = 0; o < n; o += chunk) {
    const long long k = n - o < chunk ? n - o : chunk;
    cudaError_t e = cudaMemcpy(buf.data(), src + o, 8 * k, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return scft_fail(ctx, SCFT_ERR_CUDA, cudaGetErrorString(e));
    if (fwrite(buf.data(), 8, (size_t)k, fp) != (size_t)k)
      return scft_fail(ctx, SCFT_ERR_IO, "checkpoint write failed");
  }
  return SCFT_OK;
}
int file_to_dev(scft_ctx *ctx, FILE *fp, void *dev, long long n) {
  const long long chunk = 1LL << 23;
  std::vector<uint64_t> buf((size_t)(n < chunk ? n : chunk));
  uint64_t *dst = static_cast<uint64_t *>(dev);
  for (long long o = 0; o < n; o += chunk) {
    const long long k = n - o < chunk ? n - o : chunk;
    if (fread(buf.data(), 8, (size_t)k, fp) != (size_t)k)
      return scft_fail(ctx, SCFT_ERR_IO, "checkpoint file is short");
    cudaError_t e = cudaMemcpy(dst + o, buf.data(), 8 * k, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return scft_fail(ctx, SCFT_ERR_CUDA, cudaGetErrorString(e));
  }
  return SCFT_OK;
}

bool history_kept(const scft_ctx *ctx) {
  return ctx->p.mixing == SCFT_MIX_ANDERSON && ctx->m1 > 0 &&
         (int)ctx->hist_u.size() == ctx->m1 && ctx->gram != nullptr;
}

}  // namespace

extern "C" {

int scft_save_checkpoint(scft_ctx *ctx, const char *path, int with_history) {
  if (!ctx || !path) return SCFT_ERR_INVALID_ARG;
  cudaSetDevice(ctx->p.device);
  cudaError_t e = cudaStreamSynchronize(ctx->st);
  if (e != cudaSuccess) return scft_fail(ctx, SCFT_ERR_CUDA, cudaGetErrorString(e));
  const scft_params &p = ctx->p;
  CkptHeader h;
  memset(&h, 0, sizeof h);
  memcpy(h.magic, "SCFTCKP2", 8);
  h.version = 2;
  h.nx = p.nx; h.ny = p.ny; h.nz = p.nz; h.batch = ctx->batch;
  h.precision = p.precision; h.mixing = p.mixing; h.history = p.anderson_history;
  h.has_history = (with_history && history_kept(ctx)) ? 1 : 0;
  h.lx = p.lx; h.ly = p.ly; h.lz = p.lz; h.hAB = p.hAB; h.fA = p.fA; h.ds0 = p.ds0;
  h.and_count = ctx->and_count;
  h.anderson_lambda = p.anderson_lambda;
  FILE *fp = fopen(path, "wb");
  if (!fp) return scft_fail(ctx, SCFT_ERR_IO, std::string("cannot write ") + path);
  int rc = fwrite(&h, sizeof h, 1, fp) == 1 ? SCFT_OK
                                             : scft_fail(ctx, SCFT_ERR_IO, "checkpoint write failed");
  const long long BM = ctx->M * ctx->batch;
  const double *fields[4] = {ctx->wa, ctx->wb, ctx->pha, ctx->phb};
  for (int k = 0; k < 4 && rc == SCFT_OK; ++k) rc = dev_to_file(ctx, fp, fields[k], BM);
  if (rc == SCFT_OK) rc = dev_to_file(ctx, fp, ctx->res, 4LL * ctx->batch);
  if (rc == SCFT_OK && h.has_history) {
    const int32_t m1 = ctx->m1;
    if (fwrite(&m1, sizeof m1, 1, fp) != 1) rc = scft_fail(ctx, SCFT_ERR_IO, "checkpoint write failed");
    for (int j = 0; j < m1 && rc == SCFT_OK; ++j) rc = dev_to_file(ctx, fp, ctx->hist_u[j], 2 * BM);
    for (int j = 0; j < m1 && rc == SCFT_OK; ++j) rc = dev_to_file(ctx, fp, ctx->hist_d[j], 2 * BM);
    if (rc == SCFT_OK) rc = dev_to_file(ctx, fp, ctx->gram, (long long)ctx->batch * m1 * m1);
  }
  if (fclose(fp) != 0 && rc == SCFT_OK) rc = scft_fail(ctx, SCFT_ERR_IO, "checkpoint close failed");
  return rc;
}

int scft_load_checkpoint(scft_ctx *ctx, const char *path) {
  if (!ctx || !path) return SCFT_ERR_INVALID_ARG;
  FILE *fp = fopen(path, "rb");
  if (!fp) return scft_fail(ctx, SCFT_ERR_IO, std::string("cannot open ") + path);
  auto io_fail = [&](int st, const std::string &m) {
    fclose(fp);
    return scft_fail(ctx, st, m);
  };
  CkptHeader h;
  if (fread(&h, sizeof h, 1, fp) != 1 || memcmp(h.magic, "SCFTCKP2", 8) != 0 || h.version != 2)
    return io_fail(SCFT_ERR_IO, std::string("not a checkpoint file of this version: ") + path);
  const scft_params &p = ctx->p;
  if (h.nx != p.nx || h.ny != p.ny || h.nz != p.nz || h.batch != ctx->batch)
    return io_fail(SCFT_ERR_INVALID_ARG, "checkpoint grid or batch differs from the context");
  // The whole file is checked against the size its header implies before
  // anything reaches the device, so a short or padded file leaves the
  // context's fields and history as they were.
  const long long BM = ctx->M * ctx->batch;
  const long long fields_bytes = (4 * BM + 4LL * ctx->batch) * (long long)sizeof(double);
  const long long off_m1 = (long long)sizeof h + fields_bytes;
  if (fseek(fp, 0, SEEK_END) != 0) return io_fail(SCFT_ERR_IO, "checkpoint seek failed");
  const long long size = ftell(fp);
  int32_t m1 = 0;
  long long expect = off_m1;
  if (h.has_history) {
    if (size < off_m1 + (long long)sizeof m1 || fseek(fp, off_m1, SEEK_SET) != 0 ||
        fread(&m1, sizeof m1, 1, fp) != 1)
      return io_fail(SCFT_ERR_IO, "checkpoint file is short");
    if (m1 < 2 || m1 > 64) return io_fail(SCFT_ERR_IO, "checkpoint history length is corrupt");
    expect += (long long)sizeof m1 +
              ((long long)m1 * 2 * 2 * BM + (long long)ctx->batch * m1 * m1) *
                  (long long)sizeof(double);
  }
  if (size != expect)
    return io_fail(SCFT_ERR_IO, size < expect ? "checkpoint file is short"
                                              : "checkpoint file has trailing bytes");
  // fields and residual norms through one host buffer, then to the device
  std::vector<double> host((size_t)(4 * BM + 4LL * ctx->batch));
  if (fseek(fp, (long)sizeof h, SEEK_SET) != 0 ||
      fread(host.data(), sizeof(double), host.size(), fp) != host.size())
    return io_fail(SCFT_ERR_IO, "checkpoint read failed");
  cudaSetDevice(ctx->p.device);
  cudaError_t e = cudaStreamSynchronize(ctx->st);
  if (e != cudaSuccess) return io_fail(SCFT_ERR_CUDA, cudaGetErrorString(e));
  double *fields[4] = {ctx->wa, ctx->wb, ctx->pha, ctx->phb};
  for (int k = 0; k < 4 && e == cudaSuccess; ++k)
    e = cudaMemcpy(fields[k], host.data() + k * BM, sizeof(double) * BM, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(ctx->res, host.data() + 4 * BM, sizeof(double) * 4 * ctx->batch,
                   cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return io_fail(SCFT_ERR_CUDA, cudaGetErrorString(e));
  std::vector<double>().swap(host);
  // the history restarts unless the file's ring belongs to this operator; a
  // ring only counts once it is fully copied (and_count stays 0 until then)
  ctx->and_count = 0;
  ctx->have_conc = false;   // the stored propagators belong to other fields
  int rc = SCFT_OK;
  if (h.has_history) {
    const bool same = history_kept(ctx) && h.precision == p.precision &&
                      h.mixing == p.mixing && h.history == p.anderson_history &&
                      h.lx == p.lx && h.ly == p.ly && h.lz == p.lz && h.hAB == p.hAB &&
                      h.fA == p.fA && h.ds0 == p.ds0 &&
                      h.anderson_lambda == p.anderson_lambda;
    if (same && m1 == ctx->m1 && fseek(fp, (long)(off_m1 + (long long)sizeof m1), SEEK_SET) == 0) {
      for (int j = 0; j < m1 && rc == SCFT_OK; ++j) rc = file_to_dev(ctx, fp, ctx->hist_u[j], 2 * BM);
      for (int j = 0; j < m1 && rc == SCFT_OK; ++j) rc = file_to_dev(ctx, fp, ctx->hist_d[j], 2 * BM);
      if (rc == SCFT_OK) rc = file_to_dev(ctx, fp, ctx->gram, (long long)ctx->batch * m1 * m1);
      if (rc == SCFT_OK) ctx->and_count = h.and_count;
    }
  }
  fclose(fp);
  return rc;
}

}  // extern "C"
