// scft_split_step_noalloc: one FP32 propagator split step that allocates no
// device memory.
//
// Who needs it: callers that cannot call cudaMalloc at the point where they
// advance a propagator.  For example, a host framework that owns all device
// memory through its own pool and forbids raw allocations in plug-ins, or a
// latency-critical loop where cudaMalloc's implicit device synchronisation is
// unacceptable.  They pass their own input,
// Boltzmann factor and output buffers; everything else the step needs (the
// two intermediates between the per-axis passes and the per-axis FFT tables)
// lives in the file-scope scratch array below.
//
// Limits and sharing:
//  - batch * Nx*Ny*Nz must not exceed kNoAllocMaxPoints (2^21, e.g. one 128^3
//    grid or eight 64^3 grids), batch must not exceed 65535 (the launch grid's
//    z limit); axes up to 4096 points.  Larger requests are rejected with
//    SCFT_ERR_INVALID_ARG before anything is enqueued.
//  - The array (2 * 2^21 floats + tables, about 16.2 MB) is held by every GPU
//    that loads this library, until the process exits.
//  - Every call shares the one array: two calls whose work overlaps on the GPU
//    (different streams, or different host threads) race on it.  Serialise
//    them on one stream.
//  - The first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) and sets kernel attributes, once per device under
//    a lock (host threads may race to it); make that first call before any
//    stream capture on that device.
//  - A failure is this call's own: each launch's status is read from its own
//    cudaLaunchKernelEx, never from the thread's last-error state, so an
//    earlier unrelated runtime error does not fail a valid call.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <string>

#include "ctx.h"

namespace {

constexpr long long kNoAllocMaxPoints = 1LL << 21;
constexpr int kNoAllocMaxAxis = 4096;
constexpr long long kTableFloats = 3LL * 3 * kNoAllocMaxAxis;  // per axis: twiddles (2n) + gains (n)
constexpr int kMaxDevices = 64;

// The scratch: [intermediate 0][intermediate 1][tables].  No part of it needs
// to start at zero: the tables are rewritten by every call, and each
// intermediate is fully written by one pass before the next pass reads it.
static __device__ __align__(256) float g_noalloc_scratch[2 * kNoAllocMaxPoints + kTableFloats];

// device address of the array, per device; set once under g_setup_mu
std::atomic<float *> g_scratch_dev[kMaxDevices];
std::mutex g_setup_mu;
thread_local std::string g_noalloc_err = "no error";   // per host thread

int fail(int st, const std::string &m) {
  g_noalloc_err = m;
  return st;
}

constexpr double kPiRef = 3.1415926535;  // struct.h:11

// Twiddles exp(-2 pi i m/n) and gains exp(-ds0*k_m^2)/n * scale, with the
// reference's wave numbers (init_cuda.cu:398-418), computed on the device.
__global__ void k_noalloc_tables(float *tw, float *gain, int n, double len, double ds0,
                                 double scale) {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(-2.0 * (double)m / (double)n, &s, &c);
    tw[2 * m] = (float)c;
    tw[2 * m + 1] = (float)s;
    const double d = len / n;
    const double k = m <= n / 2 - 1 ? 2 * kPiRef * m * 1.0 / n / d : 2 * kPiRef * (m - n) * 1.0 / d / n;
    gain[m] = (float)(exp(-ds0 * k * k) / n * scale);
  }
}

double k2_len1(double len) {   // the reference's bin 0 of a length-1 axis: k = -2*pi/len
  const double k = 2 * kPiRef * (0 - 1) * 1.0 / len / 1;
  return k * k;
}

}  // namespace

extern "C" const char *scft_noalloc_last_error(void) { return g_noalloc_err.c_str(); }

extern "C" int scft_split_step_noalloc(int nx, int ny, int nz, double lx, double ly, double lz,
                                       double ds0, int batch, const float *q_in, const float *W,
                                       float *q_out, void *stream) {
  if (!q_in || !W || !q_out) return fail(SCFT_ERR_INVALID_ARG, "null buffer");
  if ((reinterpret_cast<uintptr_t>(q_in) | reinterpret_cast<uintptr_t>(W) |
       reinterpret_cast<uintptr_t>(q_out)) & 15)
    return fail(SCFT_ERR_INVALID_ARG, "q_in, W and q_out must be 16-byte aligned");
  if (batch < 1 || !(lx > 0 && ly > 0 && lz > 0 && ds0 > 0))
    return fail(SCFT_ERR_INVALID_ARG, "bad batch, box or ds0");
  if (batch > 65535)
    return fail(SCFT_ERR_INVALID_ARG, "batch " + std::to_string(batch) +
                                          " exceeds the launch limit of 65535 instances");
  if (!scft_grid_supported(nx, ny, nz) || nx > kNoAllocMaxAxis || ny > kNoAllocMaxAxis ||
      nz > kNoAllocMaxAxis)
    return fail(SCFT_ERR_UNSUPPORTED, "grid not supported by the kernels");
  const long long M = (long long)nx * ny * nz;
  if (M * batch > kNoAllocMaxPoints)
    return fail(SCFT_ERR_INVALID_ARG,
                "batch*Nx*Ny*Nz = " + std::to_string(M * batch) + " exceeds the no-allocation "
                "maximum of " + std::to_string(kNoAllocMaxPoints) + " points");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(SCFT_ERR_NO_DEVICE, "no current CUDA device");
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  // once per device, with that device current (host threads may race here)
  float *scratch = g_scratch_dev[dev].load(std::memory_order_acquire);
  if (!scratch) {
    std::lock_guard<std::mutex> lock(g_setup_mu);
    scratch = g_scratch_dev[dev].load(std::memory_order_relaxed);
    if (!scratch) {
      void *p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess)
        return fail(SCFT_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      if (scft::line_filter_prepare() != cudaSuccess || scft::fast_line_prepare() != cudaSuccess)
        return fail(SCFT_ERR_CUDA, "kernel attribute set-up failed");
      scratch = static_cast<float *>(p);
      g_scratch_dev[dev].store(scratch, std::memory_order_release);
    }
  }
  float *tmp[2] = {scratch, scratch + kNoAllocMaxPoints};
  float *tables = scratch + 2 * kNoAllocMaxPoints;

  // per-axis passes, as scft_create builds them (length-1 axes fold into the first)
  const int dims[3] = {nx, ny, nz};
  const double lens[3] = {lx, ly, lz};
  double scale = 1.0;
  int axes[3], na = 0;
  for (int a = 0; a < 3; ++a) {
    if (dims[a] == 1) scale *= exp(-ds0 * k2_len1(lens[a]));
    else axes[na++] = a;
  }
  scft::AxisPlan plans[3];
  for (int i = 0; i < na; ++i) {
    const int a = axes[i], n = dims[a];
    scft::AxisPlan &ap = plans[i];
    memset(&ap, 0, sizeof(ap));
    ap.n = n;
    int m = n, k = 0;
    while (m % 4 == 0) { ap.fac[k++] = 4; m /= 4; }
    while (m % 2 == 0) { ap.fac[k++] = 2; m /= 2; }
    for (int p = 3; p <= 61 && m > 1; p += 2)
      while (m % p == 0) { ap.fac[k++] = p; m /= p; }
    ap.nfac = k;
    if (a == 0) {
      ap.s_n = 1; ap.s_pair = nx; ap.n_real = ny * nz; ap.n_outer = 1; ap.n_fast = 1;
    } else if (a == 1) {
      ap.s_n = nx; ap.s_pair = 1; ap.s_outer = (long long)nx * ny; ap.n_real = nx; ap.n_outer = nz;
    } else {
      ap.s_n = (long long)nx * ny; ap.s_pair = 1; ap.s_outer = nx; ap.n_real = nx; ap.n_outer = ny;
    }
    int tl = 65536 / (4 * n * 4);
    tl = tl > 32 ? 32 : (tl < 1 ? 1 : tl);
    const int n_pairs = (ap.n_real + 1) / 2;
    ap.tl = tl > n_pairs ? n_pairs : tl;
    ap.use_fast = scft::fast_line_supported(ap) ? 1 : 0;
    if (scft::line_filter_smem_bytes(ap, 4) > (size_t)scft::kLineSmemMax)
      return fail(SCFT_ERR_UNSUPPORTED, "line too long for shared memory");
    float *tw = tables + (long long)i * 3 * kNoAllocMaxAxis;
    float *gain = tw + 2 * kNoAllocMaxAxis;
    ap.twiddle = tw;
    ap.gain = gain;
    // The pass kernels read their tables before their dependency wait
    // (griddepcontrol.wait), overlapping the previous kernel's tail.  That is
    // safe here because every table kernel is enqueued, without the
    // programmatic-launch attribute, before the first pass: a pass can only
    // overlap the last table kernel or an earlier pass, and the first pass
    // reads the first axis's tables, which an earlier table kernel wrote (with
    // one axis, the first pass is the generic kernel, which waits first).
    // Keep the table launches ahead of every pass.
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((n + 255) / 256);
    cfg.blockDim = dim3(256);
    cfg.stream = st;
    const double len = lens[a], sc = i == 0 ? scale : 1.0;
    cudaError_t e = cudaLaunchKernelEx(&cfg, k_noalloc_tables, tw, gain, n, len, ds0, sc);
    if (e != cudaSuccess) return fail(SCFT_ERR_CUDA, cudaGetErrorString(e));
  }
  // the split step: W . D_z D_y D_x (W . q_in), one pass per axis
  for (int i = 0; i < na; ++i) {
    const float *in = i == 0 ? q_in : tmp[(i - 1) & 1];
    float *out = i == na - 1 ? q_out : tmp[i & 1];
    const float *pre = i == 0 ? W : nullptr;
    const float *post = i == na - 1 ? W : nullptr;
    cudaError_t e;
    if (plans[i].use_fast) {
      scft::PassSet<float> ps;
      memset(&ps, 0, sizeof(ps));
      ps.nset = 1;
      ps.batch = batch;
      ps.w_bs = M;
      ps.in[0] = in; ps.out[0] = out; ps.pre[0] = pre; ps.post[0] = post;
      ps.in_bs[0] = M; ps.out_bs[0] = M;
      e = scft::launch_fast_line(plans[i], ps, st);
    } else {
      e = scft::launch_line_filter<float>(plans[i], in, M, out, M, pre, post, M, batch, st);
    }
    if (e != cudaSuccess) return fail(SCFT_ERR_CUDA, cudaGetErrorString(e));
  }
  return SCFT_OK;
}
