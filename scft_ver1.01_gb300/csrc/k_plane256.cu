// x and y passes of 256 x 256 z-planes, FP32: the plane kernels of k_fast.cu
// (k_xy_plane, k_xyxy) for planes too large for one CTA's shared memory
// (256 KB).  A thread-block cluster of two CTAs holds one plane: CTA rank r
// keeps rows [128 r, 128 r + 128) in its shared memory (pitch 257).  The x
// filter runs on each CTA's own rows; the y filter of the columns
// [128 r, 128 r + 128) reads and writes the other half through distributed
// shared memory (the peer's shared memory mapped into the cluster), with
// cluster barriers between the passes.  No TMA multicast.
//
// MODE 0: one step's x+y passes (the Boltzmann factor on load and/or on
//         store), the output straight from the y filter to global memory.
// MODE 1: the fused step pair (x, y, factor -> the finished slice qout,
//         factor, y, x), as k_xyxy.
//
// A CTA never leaves while its peer may still read its half: every path ends
// after a cluster barrier that follows the last remote access.
#include <cooperative_groups.h>

#include "common.cuh"
#include "fft_reg.cuh"
#include "filter_core.cuh"
#include "kernels.h"

namespace scft {

namespace {

using namespace fcore;
namespace cg = cooperative_groups;

constexpr int kN = 256;                 // line length of both axes
constexpr int kP = 16;                  // warps per line set
constexpr int kThreads = 32 * kP;
constexpr int kHalf = kN / 2;           // rows per CTA
constexpr int kPitch = kN + 1;          // conflict-free row access by lane
constexpr size_t kHalfBytes = ((size_t)kHalf * kPitch * 4 + 127) / 128 * 128;
constexpr size_t kExOff = kHalfBytes;                           // N x 32 float2
constexpr size_t kTabOff = kExOff + (size_t)kN * 32 * 8;        // x then y tables
constexpr size_t kSmem = kTabOff + (size_t)2 * filter_table_reals<kN>() * 4;

template <int MODE>
__global__ void __launch_bounds__(kThreads, 1)
    k_plane256(AxisPlan apx, AxisPlan apy, PassSet<float> ps) {
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();   // 0 or 1
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float *half = reinterpret_cast<float *>(smem_raw);
  float2 *ex = reinterpret_cast<float2 *>(smem_raw + kExOff);
  float2 *twx = reinterpret_cast<float2 *>(smem_raw + kTabOff);
  float *gx = reinterpret_cast<float *>(twx + 2 * kN);
  float2 *twy = reinterpret_cast<float2 *>(gx + kN);
  float *gy = reinterpret_cast<float *>(twy + 2 * kN);
  const int lane = threadIdx.x & 31, p = threadIdx.x >> 5;
  const int set = (int)blockIdx.z >= ps.batch ? 1 : 0;
  const long long b = (long long)blockIdx.z - (long long)set * ps.batch;
  const long long base = (long long)(blockIdx.x >> 1) * kN * kN;   // the plane
  const float *in = ps.in[set] + b * ps.in_bs[set] + base;
  float *out = ps.out[set] + b * ps.out_bs[set] + base;
  const float *pre = ps.pre[set] ? ps.pre[set] + b * ps.w_bs + base : nullptr;
  const float *post = ps.post[set] ? ps.post[set] + b * ps.w_bs + base : nullptr;
  load_filter_tables<kN, kP>(twx, gx, reinterpret_cast<const float2 *>(apx.twiddle),
                             reinterpret_cast<const float *>(apx.gain), threadIdx.x, kThreads);
  load_filter_tables<kN, kP>(twy, gy, reinterpret_cast<const float2 *>(apy.twiddle),
                             reinterpret_cast<const float *>(apy.gain), threadIdx.x, kThreads);
  pdl_wait();   // the plane is the previous pass's output
  pdl_release();

  // this CTA's rows, with the pre factor
  const long long own = (long long)rank * kHalf * kN;
  constexpr int PER = kHalf * kN / kThreads;   // 64
  constexpr int CH = 16;
#pragma unroll 1
  for (int k0 = 0; k0 < PER; k0 += CH) {
    float r[CH];
#pragma unroll
    for (int k = 0; k < CH; ++k) r[k] = __ldg(in + own + threadIdx.x + (k0 + k) * kThreads);
#pragma unroll
    for (int k = 0; k < CH; ++k) {
      const int i = threadIdx.x + (k0 + k) * kThreads;
      float x = r[k];
      if (pre) x *= __ldg(pre + own + i);
      half[(i / kN) * kPitch + (i % kN)] = x;
    }
  }
  __syncthreads();

  // x filter of this CTA's rows (rows ra, ra + 64 packed), in place
  auto x_pass = [&]() {
#pragma unroll 1
    for (int r = 0; r < kHalf / 64; ++r) {
      float2 v[kN / kP];
      const int ra = r * 32 + lane, rb = ra + kHalf / 2;
      reg::static_for<0, kN / kP>([&](auto j_) {
        constexpr int j = decltype(j_)::value;
        const int n = p + kP * j;
        v[j] = make_float2(half[ra * kPitch + n], half[rb * kPitch + n]);
      });
      four_step<kN, kP>(v, ex, twx, gx, p, lane, 0, []() {});
      reg::static_for<0, kN / kP>([&](auto j_) {
        constexpr int j = decltype(j_)::value;
        const int n = p + kP * j;
        half[ra * kPitch + n] = v[j].x;
        half[rb * kPitch + n] = v[j].y;
      });
    }
  };
  x_pass();
  cluster.sync();   // both halves filtered along x and visible to the peer

  // y filter of the columns [128 rank, 128 rank + 128): element n of a
  // column is row n of the plane, in half n / 128 (register j < 8: rows
  // 0..127) at local row n % 128
  float *peer = cluster.map_shared_rank(half, rank ^ 1);
  float *h0 = rank == 0 ? half : peer, *h1 = rank == 0 ? peer : half;
  const int c0 = rank * kHalf;
  const float *W = post;   // MODE 1: the factor between the two steps
  float *qo = MODE == 1 ? ps.qout[set] + b * ps.qout_bs[set] + base : nullptr;
#pragma unroll 1
  for (int r = 0; r < kHalf / 64; ++r) {
    float2 v[kN / kP];
    const int ca = c0 + r * 64 + lane, cb = ca + 32;
    reg::static_for<0, kN / kP>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      const float *h = j < kN / kP / 2 ? h0 : h1;
      const int lr = p + kP * (j % (kN / kP / 2));
      v[j] = make_float2(h[lr * kPitch + ca], h[lr * kPitch + cb]);
    });
    four_step<kN, kP>(v, ex, twy, gy, p, lane, 0, []() {});
    if constexpr (MODE == 0) {
      reg::static_for<0, kN / kP>([&](auto j_) {
        constexpr int j = decltype(j_)::value;
        const int n = p + kP * j;
        float a = v[j].x, c = v[j].y;
        if (post) {
          a *= __ldg(post + n * kN + ca);
          c *= __ldg(post + n * kN + cb);
        }
        out[n * kN + ca] = a;
        out[n * kN + cb] = c;
      });
    } else {
      reg::static_for<0, kN / kP>([&](auto j_) {
        constexpr int j = decltype(j_)::value;
        const int n = p + kP * j;
        const float wa = __ldg(W + n * kN + ca), wb = __ldg(W + n * kN + cb);
        const float a = v[j].x * wa, c = v[j].y * wb;
        qo[n * kN + ca] = a;
        qo[n * kN + cb] = c;
        v[j] = make_float2(a * wa, c * wb);
      });
      four_step<kN, kP>(v, ex, twy, gy, p, lane, 0, []() {});
      reg::static_for<0, kN / kP>([&](auto j_) {
        constexpr int j = decltype(j_)::value;
        float *h = j < kN / kP / 2 ? h0 : h1;
        const int lr = p + kP * (j % (kN / kP / 2));
        h[lr * kPitch + ca] = v[j].x;
        h[lr * kPitch + cb] = v[j].y;
      });
    }
  }
  cluster.sync();   // the peer is done with this half (MODE 0: before leaving)
  if constexpr (MODE == 1) {
    x_pass();       // the x filter of step s+1 on this CTA's rows
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < PER; ++k) {
      const int i = threadIdx.x + k * kThreads;
      out[own + i] = half[(i / kN) * kPitch + (i % kN)];
    }
  }
}

template <int MODE>
cudaError_t launch_t(const AxisPlan &apx, const AxisPlan &apy, const PassSet<float> &ps,
                     cudaStream_t st) {
  const long long sets = (long long)ps.nset * ps.batch;
  if (apx.n != kN || apy.n != kN || apy.s_n != kN || apy.n_outer < 1 ||
      2LL * apy.n_outer > 0x7fffffffLL || sets < 1 || sets > 65535 || ps.desc ||
      ps.nset < 1 || ps.nset > kMaxSet)
    return cudaErrorInvalidValue;
  for (int k = 0; k < ps.nset; ++k)
    if (!ps.in[k] || !ps.out[k] || (MODE == 1 && (!ps.post[k] || !ps.qout[k])))
      return cudaErrorInvalidValue;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(2 * apy.n_outer), 1, (unsigned)sets);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = kSmem;
  cfg.stream = st;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 2;
  return cudaLaunchKernelEx(&cfg, k_plane256<MODE>, apx, apy, ps);
}

}  // namespace

bool plane256_fusable(const AxisPlan &apx, const AxisPlan &apy) {
  return apx.n_fast && !apy.n_fast && apx.n == kN && apy.n == kN && apy.s_n == kN &&
         !apy.flat_nx;
}

cudaError_t plane256_prepare() {
  cudaError_t e = cudaFuncSetAttribute(k_plane256<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kSmem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_plane256<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kSmem);
  return e;
}

cudaError_t launch_xy256(const AxisPlan &apx, const AxisPlan &apy, const PassSet<float> &ps,
                         cudaStream_t st) {
  return launch_t<0>(apx, apy, ps, st);
}

cudaError_t launch_xyxy256(const AxisPlan &apx, const AxisPlan &apy, const PassSet<float> &ps,
                           cudaStream_t st) {
  return launch_t<1>(apx, apy, ps, st);
}

}  // namespace scft
