// Register-resident per-axis line filter (FP32), the fast propagator pass.
//
// Same operator as k_line.cu (one axis of the separable split step
// exp(-k^2 ds)/N), organised as a four-step FFT with compile-time N = P*R1:
//   element n = p + P*j of a line lives in warp p, register j (R1 registers),
//   lane l holds the complex column l (two real lines packed as re/im).
//   stage 1 (registers):   DFT_R1 over j, twiddle W_N^(p*k1)
//   exchange (smem):       ex[k1][p][lane]
//   stage 2 (registers):   per k1 owned by the warp: DFT_P over p -> X[k1+R1*k2],
//                          multiply by the gain, inverse DFT_P, twiddle W_N^(-p*k1)
//   exchange back, inverse DFT_R1 over k1 -> natural order.
// Column passes (lines along y or z, stride s_n) load float2 straight from
// global memory: the 32 lanes of a warp read 64 consecutive x values (256 B,
// coalesced) per element.  The x pass stages a 64-row tile through shared
// memory (row pitch N+1 floats, conflict-free) and packs rows (l, l+32).
// The Boltzmann factor of the split step is applied on load (pre) and on
// store (post), so q makes one round trip per pass.
#include "common.cuh"
#include "fft_reg.cuh"
#include "kernels.h"

namespace scft {

namespace {

template <int N, int P, bool XP>
__global__ void __launch_bounds__(P * 32) k_fast_line(AxisPlan ap, PassSet<float> ps) {
  constexpr int R1 = N / P;
  constexpr int NT = P * 32;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *ex = reinterpret_cast<float2 *>(smem_raw);
  const int lane = threadIdx.x & 31, p = threadIdx.x >> 5;
  // blockIdx.z = set * batch + instance
  const int set = (int)blockIdx.z >= ps.batch ? 1 : 0;
  const long long b = (long long)blockIdx.z - (long long)set * ps.batch;
  const float *__restrict__ in = set ? ps.in[1] : ps.in[0];
  float *__restrict__ out = set ? ps.out[1] : ps.out[0];
  const float *__restrict__ pre = set ? ps.pre[1] : ps.pre[0];
  const float *__restrict__ post = set ? ps.post[1] : ps.post[0];
  const long long in_bs = set ? ps.in_bs[1] : ps.in_bs[0];
  const long long out_bs = set ? ps.out_bs[1] : ps.out_bs[0];
  const long long w_bs = ps.w_bs;
  // the input slice is the previous pass's output
  pdl_wait();
  pdl_release();
  const float2 *__restrict__ tw = reinterpret_cast<const float2 *>(ap.twiddle);
  const float *__restrict__ gain = reinterpret_cast<const float *>(ap.gain);
  float2 v[R1];
  long long base;

  if constexpr (XP) {
    constexpr int PITCH = N + 1;
    float *stg = reinterpret_cast<float *>(smem_raw);
    base = (long long)blockIdx.x * 64 * N;  // 64 consecutive rows of N floats
    const float *src = in + b * in_bs + base;
    const float *wsrc = pre ? pre + b * w_bs + base : nullptr;
#pragma unroll 4
    for (int i = threadIdx.x; i < 64 * N; i += NT) {
      const int r = i / N, c = i % N;
      float x = __ldg(src + i);
      if (wsrc) x *= __ldg(wsrc + i);
      stg[r * PITCH + c] = x;
    }
    __syncthreads();
    reg::static_for<0, R1>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      const int n = p + P * j;
      v[j] = make_float2(stg[lane * PITCH + n], stg[(lane + 32) * PITCH + n]);
    });
    __syncthreads();
  } else {
    base = (long long)blockIdx.y * ap.s_outer + (long long)blockIdx.x * 64 + 2 * lane;
    const float *src = in + b * in_bs + base;
    reg::static_for<0, R1>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      v[j] = __ldg(reinterpret_cast<const float2 *>(src + (long long)(p + P * j) * ap.s_n));
    });
    if (pre) {
      const float *ws = pre + b * w_bs + base;
      reg::static_for<0, R1>([&](auto j_) {
        constexpr int j = decltype(j_)::value;
        const float2 w =
            __ldg(reinterpret_cast<const float2 *>(ws + (long long)(p + P * j) * ap.s_n));
        v[j].x *= w.x;
        v[j].y *= w.y;
      });
    }
  }

  // ---- stage 1: DFT_R1 over j, twiddle, exchange
  reg::dft<R1, false>(v);
  reg::static_for<0, R1>([&](auto k_) {
    constexpr int k1 = decltype(k_)::value;
    if (k1 > 0) v[k1] = cmul(v[k1], __ldg(&tw[p * k1]));
    ex[(k1 * P + p) * 32 + lane] = v[k1];
  });
  __syncthreads();

  // ---- stage 2: DFT_P over p, gain, inverse DFT_P, conjugate twiddle
  for (int k1 = p; k1 < R1; k1 += P) {
    float2 u[P];
    reg::static_for<0, P>([&](auto q_) {
      constexpr int q = decltype(q_)::value;
      u[q] = ex[(k1 * P + q) * 32 + lane];
    });
    reg::dft<P, false>(u);
    reg::static_for<0, P>([&](auto k2_) {
      constexpr int k2 = decltype(k2_)::value;
      const float g = __ldg(&gain[k1 + R1 * k2]);
      u[k2].x *= g;
      u[k2].y *= g;
    });
    reg::dft<P, true>(u);
    reg::static_for<0, P>([&](auto q_) {
      constexpr int q = decltype(q_)::value;
      if (q > 0) u[q] = cmul(u[q], cconj(__ldg(&tw[q * k1])));
      ex[(k1 * P + q) * 32 + lane] = u[q];
    });
  }
  __syncthreads();

  // ---- inverse stage 1
  reg::static_for<0, R1>([&](auto k_) {
    constexpr int k1 = decltype(k_)::value;
    v[k1] = ex[(k1 * P + p) * 32 + lane];
  });
  reg::dft<R1, true>(v);

  if constexpr (XP) {
    constexpr int PITCH = N + 1;
    float *stg = reinterpret_cast<float *>(smem_raw);
    __syncthreads();  // every warp has read its exchange slots
    reg::static_for<0, R1>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      const int n = p + P * j;
      stg[lane * PITCH + n] = v[j].x;
      stg[(lane + 32) * PITCH + n] = v[j].y;
    });
    __syncthreads();
    float *dst = out + b * out_bs + base;
    const float *wdst = post ? post + b * w_bs + base : nullptr;
#pragma unroll 4
    for (int i = threadIdx.x; i < 64 * N; i += NT) {
      const int r = i / N, c = i % N;
      float x = stg[r * PITCH + c];
      if (wdst) x *= __ldg(wdst + i);
      dst[i] = x;
    }
  } else {
    float *dst = out + b * out_bs + base;
    const float *wdst = post ? post + b * w_bs + base : nullptr;
    reg::static_for<0, R1>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      const long long off = (long long)(p + P * j) * ap.s_n;
      float2 r = v[j];
      if (wdst) {
        const float2 w = __ldg(reinterpret_cast<const float2 *>(wdst + off));
        r.x *= w.x;
        r.y *= w.y;
      }
      *reinterpret_cast<float2 *>(dst + off) = r;
    });
  }
}

template <int N, int P, bool XP> size_t fast_smem() {
  const size_t ex = (size_t)N * 32 * sizeof(float2);
  const size_t stg = XP ? (size_t)64 * (N + 1) * sizeof(float) : 0;
  return ex > stg ? ex : stg;
}

template <int N, int P, bool XP>
cudaError_t launch_one(const AxisPlan &ap, const PassSet<float> &ps, cudaStream_t st) {
  dim3 grid(ap.n_real / 64, XP ? 1 : ap.n_outer, ps.nset * ps.batch);
  return launch_pdl(k_fast_line<N, P, XP>, grid, dim3(P * 32), fast_smem<N, P, XP>(), st, ap, ps);
}

template <int N, int P, bool XP> cudaError_t prep_one() {
  return cudaFuncSetAttribute(k_fast_line<N, P, XP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)fast_smem<N, P, XP>());
}

}  // namespace

bool fast_line_supported(const AxisPlan &ap) {
  if (ap.n != 32 && ap.n != 64 && ap.n != 128 && ap.n != 256) return false;
  return ap.n_real % 64 == 0;
}

cudaError_t fast_line_prepare() {
  cudaError_t e = cudaSuccess;
#define PREP(N, P)                                              \
  if ((e = prep_one<N, P, false>()) != cudaSuccess) return e;  \
  if ((e = prep_one<N, P, true>()) != cudaSuccess) return e;
  PREP(32, 4)
  PREP(64, 8)
  PREP(128, 8)
  PREP(256, 16)
#undef PREP
  return e;
}

cudaError_t launch_fast_line(const AxisPlan &ap, const PassSet<float> &ps, cudaStream_t st) {
  if (ps.nset < 1 || ps.nset > kMaxSet) return cudaErrorInvalidValue;
  const bool xp = ap.n_fast != 0;
  switch (ap.n) {
    case 32: return xp ? launch_one<32, 4, true>(ap, ps, st) : launch_one<32, 4, false>(ap, ps, st);
    case 64: return xp ? launch_one<64, 8, true>(ap, ps, st) : launch_one<64, 8, false>(ap, ps, st);
    case 128:
      return xp ? launch_one<128, 8, true>(ap, ps, st) : launch_one<128, 8, false>(ap, ps, st);
    case 256:
      return xp ? launch_one<256, 16, true>(ap, ps, st) : launch_one<256, 16, false>(ap, ps, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace scft
