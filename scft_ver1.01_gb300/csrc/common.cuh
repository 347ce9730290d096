// Shared device/host helpers for the SCFT GB300 kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "dfloat.cuh"

namespace scft {

// Complex type matched to the working real type.
template <typename R> struct cplx;
template <> struct cplx<float> { typedef float2 type; };
template <> struct cplx<double> { typedef double2 type; };
template <> struct cplx<dfloat> { typedef dfloat2 type; };

template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
// double-float complex product: each part one dot product of pairs
__host__ __device__ __forceinline__ dfloat2 cmul(dfloat2 a, dfloat2 b) {
  dfloat2 r;
  r.x = df_dot2(a.x, b.x, a.y, -b.y);
  r.y = df_dot2(a.x, b.y, a.y, b.x);
  return r;
}
template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) {
  C r; r.x = a.x + b.x; r.y = a.y + b.y; return r;
}
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) {
  C r; r.x = a.x - b.x; r.y = a.y - b.y; return r;
}
// multiply by -i
template <typename C> __host__ __device__ __forceinline__ C cmul_mi(C a) {
  C r; r.x = a.y; r.y = -a.x; return r;
}
template <typename C, typename R> __host__ __device__ __forceinline__ C cscale(C a, R s) {
  C r; r.x = a.x * s; r.y = a.y * s; return r;
}
template <typename C> __host__ __device__ __forceinline__ C cconj(C a) {
  C r; r.x = a.x; r.y = -a.y; return r;
}
template <typename C, typename R> __host__ __device__ __forceinline__ C mkc(R x, R y) {
  C r; r.x = x; r.y = y; return r;
}

// Programmatic dependent launch.  A kernel launched with launch_pdl may start
// while its predecessor in the stream is still running; it must call
// pdl_wait() before touching anything the predecessor writes, and releases
// its own dependents with pdl_release().
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// pdl false: an ordinary stream-ordered launch of the same kernel (its
// griddepcontrol instructions then return at once).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(bool pdl, void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem,
                            cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k, args...);
}
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem,
                              cudaStream_t st, Args... args) {
  return launch_k(true, k, grid, block, smem, st, args...);
}

// Warp-level sum of a double.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Four doubles of one grid point (w_A, w_B, phi_A, phi_B) held in registers.
struct dquad {
  double x, y, z, w;
};

// Grid-stride loop over [0, n) for streaming kernels, U elements per thread
// per trip: the elements i0, i0+S, ..., i0+(U-1)S (S = the grid's thread
// count) are loaded first, load(i), then used, use(i, value).  The U loads of
// a trip are independent, so a thread keeps U requests in flight instead of
// one (a kernel with one outstanding load per thread reaches only a fraction
// of HBM bandwidth).  Consecutive threads still touch consecutive elements.
template <int U, typename L, typename F>
__device__ __forceinline__ void stream_loop(long long n, L &&load, F &&use) {
  typedef decltype(load(0LL)) V;
  const long long S = (long long)gridDim.x * blockDim.x;
  for (long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; i0 < n; i0 += U * S) {
    V v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const long long i = i0 + u * S;
      if (i < n) v[u] = load(i);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const long long i = i0 + u * S;
      if (i < n) use(i, v[u]);
    }
  }
}

// Error-free transformation a+b = s+e (Knuth TwoSum), FP32.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

}  // namespace scft
