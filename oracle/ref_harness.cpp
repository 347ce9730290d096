// Reference harness (TEST INFRASTRUCTURE ONLY): runs the reference's own CUDA
// kernels -- compiled unchanged from cuda_aid.cu / cuda_aid.cuh into
// oracle/_ref/ref_kernels.cubin -- with cuFFT D2Z/Z2D, in the order and with
// the launch shapes of the reference's host code, which is restated here:
//   setup            initialize_cufft       init_cuda.cu:296-546 (one GPU)
//   average_value    cuda_scft.cu:14-59
//   sovDifFft        cuda_scft.cu:435-563
//   getConc          cuda_scft.cu:61-138
//   Free loop body   cuda_scft.cu:167-223   (phi_w + host free energy)
// Its outputs pin the CPU oracle (tests/golden/ref_*.npz) and give the
// reference's own GPU speed on GB300.  Plain cudaMalloc replaces the
// reference's cudaMallocManaged; nothing else differs.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

namespace {

constexpr double kPiRef = 3.1415926535;  // struct.h:11

struct Ref {
  int nx = 0, ny = 0, nz = 0, nxh1 = 0, batch = 0, NsA = 0, dNsB = 0;
  long long M = 0, Mh = 0;
  double lx = 0, ly = 0, lz = 0, hAB = 0, fA = 0, ds0 = 0, ds2 = 0;
  int thread = 1, thread_sur = 1;
  CUmodule mod = nullptr;
  CUfunction f_wdz, f_q, f_qinv, f_in_go, f_sur_go, f_in_to_g_go, f_qint_init, f_qa_to_qint,
      f_qa_to_qint2, f_cal_ql, f_w_to_phi_go, f_minus_average, f_phi_w, f_reduce3,
      f_phi_w_con, f_phi_w_con_ex;
  cufftHandle plan_f = 0, plan_b = 0;
  double *kxyzdz = nullptr, *wa = nullptr, *wb = nullptr, *pha = nullptr, *phb = nullptr,
         *qint = nullptr, *wdz = nullptr, *qa = nullptr, *qca = nullptr, *qb = nullptr,
         *qcb = nullptr, *ql = nullptr, *ffl = nullptr, *in = nullptr, *sum = nullptr,
         *target = nullptr;
  cufftDoubleComplex *out = nullptr;
  std::vector<double> hql, hql_raw;
  int q_mode = 1;
  std::string err = "no error";
};

Ref g;

// init_cuda.cu:24-80 computes the largest divisor of N that is <= 1024.
int largest_divisor_1024(long long n) {
  int best = 1;
  for (int d = 1; d <= 1024 && d <= n; ++d)
    if (n % d == 0) best = d;
  return best;
}

int fail(const std::string &m) {
  g.err = m;
  return 1;
}

#define CU(x)                                                      \
  do {                                                             \
    CUresult r_ = (x);                                             \
    if (r_ != CUDA_SUCCESS) {                                      \
      const char *s_ = nullptr;                                    \
      cuGetErrorString(r_, &s_);                                   \
      return fail(std::string(#x) + ": " + (s_ ? s_ : "?"));       \
    }                                                              \
  } while (0)
#define CR(x)                                                      \
  do {                                                             \
    cudaError_t r_ = (x);                                          \
    if (r_ != cudaSuccess)                                         \
      return fail(std::string(#x) + ": " + cudaGetErrorString(r_)); \
  } while (0)
#define CF(x)                                                      \
  do {                                                             \
    cufftResult r_ = (x);                                          \
    if (r_ != CUFFT_SUCCESS) return fail(std::string(#x) + " failed"); \
  } while (0)

int find_kernel(const char *needle, CUfunction *out) {
  unsigned int n = 0;
  CU(cuModuleGetFunctionCount(&n, g.mod));
  std::vector<CUfunction> fs(n);
  CU(cuModuleEnumerateFunctions(fs.data(), n, g.mod));
  for (CUfunction f : fs) {
    const char *name = nullptr;
    CU(cuFuncGetName(&name, f));
    if (name && strstr(name, needle)) {
      *out = f;
      return 0;
    }
  }
  return fail(std::string("kernel not found: ") + needle);
}

int launch(CUfunction f, dim3 grid, dim3 block, unsigned smem, void **args) {
  CU(cuLaunchKernel(f, grid.x, grid.y, grid.z, block.x, block.y, block.z, smem, 0, args, nullptr));
  return 0;
}

// average_value, cuda_scft.cu:14-59
int average_value(double *data) {
  int threads = g.thread;
  unsigned smem = (threads <= 32) ? 2 * threads * sizeof(double) : threads * sizeof(double);
  unsigned n = (unsigned)g.M;
  void *a1[] = {&data, &g.sum, &n};
  if (launch(g.f_reduce3, dim3(g.batch), dim3(threads), smem, a1)) return 1;
  void *a2[] = {&data, &g.sum};
  if (launch(g.f_minus_average, dim3(g.nx, g.ny, g.nz), dim3(g.batch), 0, a2)) return 1;
  CR(cudaDeviceSynchronize());
  return 0;
}

// sovDifFft, cuda_scft.cu:435-563
int sov_dif_fft(double *gq, double *w, int ns, int sign) {
  int ns1 = ns + 1;
  dim3 grid(g.nx, g.ny, g.nz), block(g.batch, 1, 1);
  void *a_wdz[] = {&w, &g.wdz, &g.ds2};
  if (launch(g.f_wdz, grid, block, 0, a_wdz)) return 1;
  dim3 gridgo((unsigned)(g.M / g.thread), g.batch);
  dim3 gridgo_sur((unsigned)(g.Mh / g.thread_sur), g.batch);
  int nxh1 = g.nxh1, nx = g.nx, ny = g.ny, nz = g.nz;
  if (sign == 1) {
    void *a_q[] = {&gq, &g.qint, &ns1};
    if (launch(g.f_q, grid, block, 0, a_q)) return 1;
    for (int iz = 1; iz <= ns; iz++) {
      void *a_in[] = {&g.in, &gq, &g.wdz, &ns1, &iz};
      if (launch(g.f_in_go, gridgo, dim3(g.thread), 0, a_in)) return 1;
      CF(cufftExecD2Z(g.plan_f, g.in, g.out));
      void *a_s[] = {&g.out, &g.kxyzdz, &nxh1, &nx, &ny, &nz};
      if (launch(g.f_sur_go, gridgo_sur, dim3(g.thread_sur), 0, a_s)) return 1;
      CF(cufftExecZ2D(g.plan_b, g.out, g.in));
      void *a_g[] = {&gq, &g.wdz, &g.in, &ns1, &iz};
      if (launch(g.f_in_to_g_go, gridgo, dim3(g.thread), 0, a_g)) return 1;
      CR(cudaDeviceSynchronize());
    }
  } else {
    void *a_q[] = {&gq, &g.qint, &ns1};
    if (launch(g.f_qinv, grid, block, 0, a_q)) return 1;
    for (int iz = ns - 1; iz >= 0; iz--) {
      int izp2 = iz + 2;
      void *a_in[] = {&g.in, &gq, &g.wdz, &ns1, &izp2};
      if (launch(g.f_in_go, gridgo, dim3(g.thread), 0, a_in)) return 1;
      CF(cufftExecD2Z(g.plan_f, g.in, g.out));
      void *a_s[] = {&g.out, &g.kxyzdz, &nxh1, &nx, &ny, &nz};
      if (launch(g.f_sur_go, gridgo_sur, dim3(g.thread_sur), 0, a_s)) return 1;
      CF(cufftExecZ2D(g.plan_b, g.out, g.in));
      void *a_g[] = {&gq, &g.wdz, &g.in, &ns1, &iz};
      if (launch(g.f_in_to_g_go, gridgo, dim3(g.thread), 0, a_g)) return 1;
      CR(cudaDeviceSynchronize());
    }
  }
  CR(cudaDeviceSynchronize());
  return 0;
}

// getConc, cuda_scft.cu:61-138
int get_conc() {
  dim3 grid(g.nx, g.ny, g.nz);
  if (average_value(g.wa)) return 1;
  void *a0[] = {&g.qint};
  if (launch(g.f_qint_init, grid, dim3(g.batch), 0, a0)) return 1;
  CR(cudaDeviceSynchronize());
  if (sov_dif_fft(g.qa, g.wa, g.NsA, 1)) return 1;
  if (sov_dif_fft(g.qcb, g.wb, g.dNsB, -1)) return 1;
  void *a1[] = {&g.qint, &g.qa, &g.NsA};
  if (launch(g.f_qa_to_qint, grid, dim3(g.batch), 0, a1)) return 1;
  if (sov_dif_fft(g.qb, g.wb, g.dNsB, 1)) return 1;
  void *a2[] = {&g.qint, &g.qcb, &g.dNsB};
  if (launch(g.f_qa_to_qint2, grid, dim3(g.batch), 0, a2)) return 1;
  CR(cudaDeviceSynchronize());
  if (sov_dif_fft(g.qca, g.wa, g.NsA, -1)) return 1;
  int threads = 512;
  unsigned smem = threads * sizeof(double) * 2;
  int M = (int)g.M;
  void *a3[] = {&g.ql, &g.qb, &g.dNsB, &M};
  if (launch(g.f_cal_ql, dim3(g.batch), dim3(threads), smem, a3)) return 1;
  CR(cudaDeviceSynchronize());
  std::vector<double> ql(g.batch), ffl(g.batch);
  CR(cudaMemcpy(ql.data(), g.ql, sizeof(double) * g.batch, cudaMemcpyDeviceToHost));
  g.hql_raw = ql;
  // cal_ql stores each thread's partial (cuda_aid.cu:145) and starts the
  // shared-memory tree (:149-158) without a barrier in between, so warps can
  // read other warps' slots before they are written.  q_mode 1 replaces its
  // result by the FP64 sum of the same slice qB[.][dNsB] (what cal_ql is meant
  // to return); q_mode 0 keeps the kernel's value.
  if (g.q_mode == 1) {
    const long long ns1 = g.dNsB + 1;
    std::vector<double> all(g.M * g.batch * ns1);
    CR(cudaMemcpy(all.data(), g.qb, sizeof(double) * all.size(), cudaMemcpyDeviceToHost));
    for (int i = 0; i < g.batch; i++) {
      double s = 0.0;
      for (long long r = 0; r < g.M; ++r) s += all[(r * ns1 + g.dNsB) + i * g.M * ns1];
      ql[i] = s;
    }
  }
  for (int i = 0; i < g.batch; i++) {
    ql[i] /= g.M;
    ffl[i] = g.ds0 / ql[i];
  }
  g.hql = ql;
  CR(cudaMemcpy(g.ql, ql.data(), sizeof(double) * g.batch, cudaMemcpyHostToDevice));
  CR(cudaMemcpy(g.ffl, ffl.data(), sizeof(double) * g.batch, cudaMemcpyHostToDevice));
  dim3 gridgo((unsigned)(g.M / g.thread), g.batch);
  void *a4[] = {&g.pha, &g.phb, &g.qa, &g.qca, &g.qb, &g.qcb, &g.NsA, &g.dNsB, &g.ffl};
  if (launch(g.f_w_to_phi_go, gridgo, dim3(g.thread), 0, a4)) return 1;
  CR(cudaDeviceSynchronize());
  return 0;
}

int phi_w() {
  void *a[] = {&g.wa, &g.wb, &g.pha, &g.phb, &g.hAB};
  if (launch(g.f_phi_w, dim3(g.nx, g.ny, g.nz), dim3(g.batch), 0, a)) return 1;
  CR(cudaDeviceSynchronize());
  return 0;
}

// phi_w_constrained / phi_w_constrainedEx (cuda_aid.cu:418-490), launched
// with phi_w's geometry; the reference has no call site for them.
int phi_w_constrained(int ex, double lambda) {
  if (!g.target) return fail("no target field");
  void *a[] = {&g.wa, &g.wb, &g.pha, &g.phb, &g.target, &g.hAB, &lambda};   // Ex: no lambda
  void *a_ex[] = {&g.wa, &g.wb, &g.pha, &g.phb, &g.target, &g.hAB};
  if (launch(ex ? g.f_phi_w_con_ex : g.f_phi_w_con, dim3(g.nx, g.ny, g.nz), dim3(g.batch), 0,
             ex ? a_ex : a))
    return 1;
  CR(cudaDeviceSynchronize());
  return 0;
}

void release() {
  cudaFree(g.kxyzdz); cudaFree(g.wa); cudaFree(g.wb); cudaFree(g.pha); cudaFree(g.phb);
  cudaFree(g.qint); cudaFree(g.wdz); cudaFree(g.qa); cudaFree(g.qca); cudaFree(g.qb);
  cudaFree(g.qcb); cudaFree(g.ql); cudaFree(g.ffl); cudaFree(g.in); cudaFree(g.out);
  cudaFree(g.sum); cudaFree(g.target);
  if (g.plan_f) cufftDestroy(g.plan_f);
  if (g.plan_b) cufftDestroy(g.plan_b);
  if (g.mod) cuModuleUnload(g.mod);
  std::string e = g.err;
  g = Ref();
  g.err = e;
}

}  // namespace

extern "C" {

const char *ref_last_error() { return g.err.c_str(); }

// initialize_cufft (init_cuda.cu:296-546) for one GPU.
int ref_open(const char *cubin, int nx, int ny, int nz, double lx, double ly, double lz,
             double hAB, double fA, double ds0, int batch) {
  release();
  g.nx = nx; g.ny = ny; g.nz = nz; g.lx = lx; g.ly = ly; g.lz = lz;
  g.hAB = hAB; g.fA = fA; g.ds0 = ds0; g.batch = batch;
  g.M = (long long)nx * ny * nz;
  g.nxh1 = nx / 2 + 1;
  g.Mh = (long long)g.nxh1 * ny * nz;
  g.thread = largest_divisor_1024(g.M);
  g.thread_sur = largest_divisor_1024(g.Mh);
  g.ds2 = ds0 / 2;
  g.NsA = (int)(fA / ds0 + 1.0e-8);
  g.dNsB = (int)((1 - fA) / ds0 + 1.0e-8);
  CR(cudaSetDevice(0));
  CR(cudaFree(0));   // create the primary context used by cuFFT and the module
  CU(cuModuleLoad(&g.mod, cubin));
  struct { const char *n; CUfunction *f; } ks[] = {
      {"initilize_wdz", &g.f_wdz}, {"11initilize_qPd", &g.f_q},
      {"initilize_q_inverse", &g.f_qinv}, {"initilize_in_go", &g.f_in_go},
      {"sufaceField_go", &g.f_sur_go}, {"in_to_g_go", &g.f_in_to_g_go},
      {"qInt_init", &g.f_qint_init}, {"10qa_to_qInt", &g.f_qa_to_qint},
      {"qa_to_qInt2", &g.f_qa_to_qint2}, {"cal_ql", &g.f_cal_ql},
      {"w_to_phi_go", &g.f_w_to_phi_go}, {"minus_average", &g.f_minus_average},
      {"5phi_w", &g.f_phi_w}, {"reduce3", &g.f_reduce3},
      {"17phi_w_constrained", &g.f_phi_w_con}, {"19phi_w_constrainedEx", &g.f_phi_w_con_ex}};
  for (auto &k : ks)
    if (find_kernel(k.n, k.f)) return 1;
  int dim[3] = {nz, ny, nx};   // init_cuda.cu:345
  CF(cufftPlanMany(&g.plan_f, 3, dim, NULL, 1, 1, NULL, 1, 1, CUFFT_D2Z, batch));
  CF(cufftPlanMany(&g.plan_b, 3, dim, NULL, 1, 1, NULL, 1, 1, CUFFT_Z2D, batch));
  // kxyzdz table, init_cuda.cu:394-428
  std::vector<double> kx(nx), ky(ny), kz(nz), tab(g.M);
  double dx = lx / nx, dy = ly / ny, dz = lz / nz;
  for (int i = 0; i <= nx / 2 - 1; i++) kx[i] = 2 * kPiRef * i * 1.0 / nx / dx;
  for (int i = nx / 2; i < nx; i++) kx[i] = 2 * kPiRef * (i - nx) * 1.0 / dx / nx;
  for (int i = 0; i < nx; i++) kx[i] *= kx[i];
  for (int i = 0; i <= ny / 2 - 1; i++) ky[i] = 2 * kPiRef * i * 1.0 / ny / dy;
  for (int i = ny / 2; i < ny; i++) ky[i] = 2 * kPiRef * (i - ny) * 1.0 / dy / ny;
  for (int i = 0; i < ny; i++) ky[i] *= ky[i];
  for (int i = 0; i <= nz / 2 - 1; i++) kz[i] = 2 * kPiRef * i * 1.0 / nz / dz;
  for (int i = nz / 2; i < nz; i++) kz[i] = 2 * kPiRef * (i - nz) * 1.0 / dz / nz;
  for (int i = 0; i < nz; i++) kz[i] *= kz[i];
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        long long ijk = (long long)((k * ny + j) * nx + i);
        double ksq = kx[i] + ky[j] + kz[k];
        tab[ijk] = exp(-ds0 * ksq);
      }
  const long long M = g.M, B = batch;
  CR(cudaMalloc(&g.kxyzdz, sizeof(double) * M));
  CR(cudaMemcpy(g.kxyzdz, tab.data(), sizeof(double) * M, cudaMemcpyHostToDevice));
  CR(cudaMalloc(&g.wa, sizeof(double) * M * B));
  CR(cudaMalloc(&g.wb, sizeof(double) * M * B));
  CR(cudaMalloc(&g.pha, sizeof(double) * M * B));
  CR(cudaMalloc(&g.phb, sizeof(double) * M * B));
  CR(cudaMalloc(&g.qint, sizeof(double) * M * B));
  CR(cudaMalloc(&g.wdz, sizeof(double) * M * B));
  CR(cudaMalloc(&g.qa, sizeof(double) * M * B * (g.NsA + 1)));
  CR(cudaMalloc(&g.qca, sizeof(double) * M * B * (g.NsA + 1)));
  CR(cudaMalloc(&g.qb, sizeof(double) * M * B * (g.dNsB + 1)));
  CR(cudaMalloc(&g.qcb, sizeof(double) * M * B * (g.dNsB + 1)));
  CR(cudaMalloc(&g.ql, sizeof(double) * B));
  CR(cudaMalloc(&g.ffl, sizeof(double) * B));
  CR(cudaMalloc(&g.sum, sizeof(double) * B));
  CR(cudaMalloc(&g.in, sizeof(double) * M * B));
  CR(cudaMalloc(&g.out, sizeof(cufftDoubleComplex) * g.Mh * B));
  CR(cudaMemset(g.pha, 0, sizeof(double) * M * B));
  CR(cudaMemset(g.phb, 0, sizeof(double) * M * B));
  g.hql.assign(B, 0.0);
  return 0;
}

void ref_close() { release(); }

int ref_get_ns(int *NsA, int *dNsB) {
  *NsA = g.NsA;
  *dNsB = g.dNsB;
  return 0;
}

// which: 0 wa, 1 wb, 2 pha, 3 phb
int ref_set_field(int which, const double *src) {
  double *d[4] = {g.wa, g.wb, g.pha, g.phb};
  if (which < 0 || which > 3) return fail("bad field");
  CR(cudaMemcpy(d[which], src, sizeof(double) * g.M * g.batch, cudaMemcpyHostToDevice));
  return 0;
}
int ref_get_field(int which, double *dst) {
  double *d[4] = {g.wa, g.wb, g.pha, g.phb};
  if (which < 0 || which > 3) return fail("bad field");
  CR(cudaMemcpy(dst, d[which], sizeof(double) * g.M * g.batch, cudaMemcpyDeviceToHost));
  return 0;
}
// Q per instance (ql/M after getConc)
int ref_get_Q(double *dst) {
  for (int i = 0; i < g.batch; ++i) dst[i] = g.hql[i];
  return 0;
}
// The raw cal_ql kernel result (sum, not divided by M) of the last getConc.
int ref_get_ql_raw(double *dst) {
  for (int i = 0; i < g.batch && i < (int)g.hql_raw.size(); ++i) dst[i] = g.hql_raw[i];
  return 0;
}
// 0: use cal_ql's value as the reference does; 1 (default): FP64 sum of the
// same qB slice (see get_conc).
int ref_set_q_mode(int mode) {
  g.q_mode = mode;
  return 0;
}
// Runs the reference's cal_ql kernel `n` times back to back on the current
// qB and returns each raw result for instance 0 (race diagnostics).
int ref_cal_ql_repeat(int n, double *dst) {
  int threads = 512;
  unsigned smem = threads * sizeof(double) * 2;
  int M = (int)g.M;
  void *a3[] = {&g.ql, &g.qb, &g.dNsB, &M};
  for (int k = 0; k < n; ++k) {
    if (launch(g.f_cal_ql, dim3(g.batch), dim3(threads), smem, a3)) return 1;
    CR(cudaDeviceSynchronize());
    CR(cudaMemcpy(&dst[k], g.ql, sizeof(double), cudaMemcpyDeviceToHost));
  }
  return 0;
}
// slice s of propagator which (0 qa, 1 qcb, 2 qb, 3 qca) as [batch][M]; the
// reference layout is g[b][r][s] (cuda_aid.cu:237)
int ref_get_q(int which, int s, double *dst) {
  double *q[4] = {g.qa, g.qcb, g.qb, g.qca};
  int ns[4] = {g.NsA, g.dNsB, g.dNsB, g.NsA};
  if (which < 0 || which > 3 || s < 0 || s > ns[which]) return fail("bad propagator");
  const long long ns1 = ns[which] + 1;
  std::vector<double> all(g.M * g.batch * ns1);
  CR(cudaMemcpy(all.data(), q[which], sizeof(double) * all.size(), cudaMemcpyDeviceToHost));
  for (long long b = 0; b < g.batch; ++b)
    for (long long r = 0; r < g.M; ++r) dst[b * g.M + r] = all[(r * ns1 + s) + b * g.M * ns1];
  return 0;
}
int ref_average_value(int which) { return average_value(which == 0 ? g.wa : g.wb); }
int ref_get_conc() { return get_conc(); }
int ref_phi_w() { return phi_w(); }
int ref_set_target(const double *src) {
  if (!g.target) CR(cudaMalloc(&g.target, sizeof(double) * g.M * g.batch));
  CR(cudaMemcpy(g.target, src, sizeof(double) * g.M * g.batch, cudaMemcpyHostToDevice));
  return 0;
}
int ref_phi_w_constrained(int ex, double lambda) { return phi_w_constrained(ex, lambda); }

// n iterations of the Free loop body (cuda_scft.cu:167-186); after the last
// one, the free-energy block (:190-221) on the host: out5[b] = {F, FAB, FW, FS, inc}.
int ref_iterate(int n, double *out5) {
  for (int it = 0; it < n; ++it) {
    if (average_value(g.wa) || average_value(g.wb) || get_conc() || phi_w()) return 1;
  }
  if (out5) {
    const long long M = g.M;
    std::vector<double> a(M * g.batch), b(M * g.batch), pa(M * g.batch), pb(M * g.batch);
    CR(cudaMemcpy(a.data(), g.wa, sizeof(double) * a.size(), cudaMemcpyDeviceToHost));
    CR(cudaMemcpy(b.data(), g.wb, sizeof(double) * b.size(), cudaMemcpyDeviceToHost));
    CR(cudaMemcpy(pa.data(), g.pha, sizeof(double) * a.size(), cudaMemcpyDeviceToHost));
    CR(cudaMemcpy(pb.data(), g.phb, sizeof(double) * a.size(), cudaMemcpyDeviceToHost));
    for (int i = 0; i < g.batch; i++) {
      double fW = 0, fAB = 0, inc = 0;
      for (long long ijk = 0; ijk < M; ijk++) {
        const long long o = ijk + i * M;
        double ps = fabs(1 - pa[o] - pb[o]);
        if (ps > inc) inc = ps;
        fAB = fAB + g.hAB * pa[o] * pb[o];
        fW = fW - (a[o] * pa[o] + b[o] * pb[o]);
      }
      fAB /= M;
      fW /= M;
      double fS = -log(g.hql[i]);
      out5[5 * i + 0] = fAB + fW + fS;
      out5[5 * i + 1] = fAB;
      out5[5 * i + 2] = fW;
      out5[5 * i + 3] = fS;
      out5[5 * i + 4] = inc;
    }
  }
  return 0;
}

// fft_test-style timing (cuda_scft.cu:411-425) of n loop-body iterations.
int ref_time_iterations(int n, double *ms) {
  cudaEvent_t a, b;
  CR(cudaEventCreate(&a));
  CR(cudaEventCreate(&b));
  CR(cudaEventRecord(a, 0));
  int rc = ref_iterate(n, nullptr);
  CR(cudaEventRecord(b, 0));
  CR(cudaEventSynchronize(b));
  float f = 0;
  CR(cudaEventElapsedTime(&f, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = f;
  return rc;
}

}  // extern "C"
