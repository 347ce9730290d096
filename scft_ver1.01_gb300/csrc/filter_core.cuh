// The four-step line filter core shared by the register-resident pass
// kernels (k_fast.cu) and the persistent march engine (k_engine.cu): one
// axis of the separable split-step operator, IFFT . diag(g) . FFT along lines
// of compile-time length N = P * R1 held in registers (element p + P*j of a
// line in warp p, register j; lane l holds complex line l), with one
// shared-memory exchange per transform direction.
#pragma once

#include <type_traits>

#include "common.cuh"
#include "fft_reg.cuh"

namespace scft {
namespace fcore {

// The four-step filter core (FP32 or FP64 complex C, real T): v[j] holds
// element p + P*j of complex column `lane` on entry and the filtered values
// on exit.  `after_first_sync` runs once every warp has written its stage-1
// exchange slots (so every warp has finished reading its inputs).
// bar_id 0 synchronises the whole CTA; bar_id > 0 only the P warps of one
// warp group (named barrier bar_id), so several groups can filter
// independent line sets in one CTA.
__device__ __forceinline__ void group_sync(int bar_id, int nthreads) {
  if (bar_id == 0) __syncthreads();
  else asm volatile("bar.sync %0, %1;" ::"r"(bar_id), "r"(nthreads) : "memory");
}

// The tables four_step reads, laid out so that every access is a constant
// offset from one per-thread base (shared memory, 16-byte aligned):
//   tw[p*R1 + k1]     = W_N^(p*k1)          stage-1 twiddles of warp p
//   tw[N + k1*P + q]  = conj(W_N^(q*k1))    stage-2 inverse twiddles of column k1
//   gain[k1*P + k2]   = g[k1 + R1*k2]       the filter gain at X[k1 + R1*k2]
// built from the natural tables tw_n[m] = W_N^m, g_n[m] (global memory) by
// load_filter_tables.  (four_step_compact keeps the natural layout.)
template <int N, int P, typename C, typename T>
__device__ __forceinline__ void load_filter_tables(C *tw, T *gain, const C *tw_n, const T *g_n,
                                                   int tid, int nthreads) {
  constexpr int R1 = N / P;
  for (int i = tid; i < N; i += nthreads) {
    const int p = i / R1, k1 = i % R1;
    tw[i] = ldg(tw_n + (p * k1) % N);
    const int c = i / P, q = i % P;
    tw[N + i] = cconj(ldg(tw_n + (q * c) % N));
    gain[i] = ldg(g_n + c + R1 * q);
  }
}
// The natural tables (four_step_compact).
template <int N, typename C, typename T>
__device__ __forceinline__ void load_natural_tables(C *tw, T *gain, const C *tw_n, const T *g_n,
                                                    int tid, int nthreads) {
  for (int i = tid; i < N; i += nthreads) {
    tw[i] = ldg(tw_n + i);
    gain[i] = ldg(g_n + i);
  }
}
// Shared-memory reals the tables of a length-N filter take (either layout).
template <int N> constexpr int filter_table_reals() { return 5 * N; }

// Two consecutive complex table entries (one 16-byte load for FP32), and four
// consecutive gains (one 16-byte load for FP32).
template <typename C> __device__ __forceinline__ void ld_c2(const C *a, C &x, C &y) {
  if constexpr (sizeof(C) == 8) {
    const float4 t = *reinterpret_cast<const float4 *>(a);
    x.x = t.x; x.y = t.y; y.x = t.z; y.y = t.w;
  } else {
    x = a[0];
    y = a[1];
  }
}
template <typename T> __device__ __forceinline__ void ld_r4(const T *a, T (&r)[4]) {
  if constexpr (sizeof(T) == 4) {
    const float4 t = *reinterpret_cast<const float4 *>(a);
    r[0] = t.x; r[1] = t.y; r[2] = t.z; r[3] = t.w;
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i) r[i] = a[i];
  }
}

template <int N, int P, typename C, typename T, typename F>
__device__ __forceinline__ void four_step(C (&v)[N / P], C *ex, const C *tw, const T *gain, int p,
                                          int lane, int bar_id, F &&after_first_sync) {
  constexpr int R1 = N / P;
  static_assert(R1 % 2 == 0 && P % 4 == 0, "table vector loads");
  reg::dft<R1, false>(v);
  const C *t1 = tw + p * R1;
  reg::static_for<0, R1 / 2>([&](auto h_) {
    constexpr int k1 = 2 * decltype(h_)::value;
    C wa, wb;
    ld_c2(t1 + k1, wa, wb);
    if (k1 > 0) v[k1] = cmul(v[k1], wa);
    v[k1 + 1] = cmul(v[k1 + 1], wb);
    ex[(k1 * P + p) * 32 + lane] = v[k1];
    ex[((k1 + 1) * P + p) * 32 + lane] = v[k1 + 1];
  });
  group_sync(bar_id, P * 32);
  after_first_sync();
  for (int k1 = p; k1 < R1; k1 += P) {
    C u[P];
    reg::static_for<0, P>([&](auto q_) {
      constexpr int q = decltype(q_)::value;
      u[q] = ex[(k1 * P + q) * 32 + lane];
    });
    reg::dft<P, false>(u);
    const T *gk = gain + k1 * P;
    reg::static_for<0, P / 4>([&](auto h_) {
      constexpr int k2 = 4 * decltype(h_)::value;
      T g[4];
      ld_r4(gk + k2, g);
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        u[k2 + i].x *= g[i];
        u[k2 + i].y *= g[i];
      }
    });
    reg::dft<P, true>(u);
    const C *t2 = tw + N + k1 * P;
    reg::static_for<0, P / 2>([&](auto h_) {
      constexpr int q = 2 * decltype(h_)::value;
      C wa, wb;
      ld_c2(t2 + q, wa, wb);
      if (q > 0) u[q] = cmul(u[q], wa);
      u[q + 1] = cmul(u[q + 1], wb);
      ex[(k1 * P + q) * 32 + lane] = u[q];
      ex[(k1 * P + q + 1) * 32 + lane] = u[q + 1];
    });
  }
  group_sync(bar_id, P * 32);
  reg::static_for<0, R1>([&](auto k_) {
    constexpr int k1 = decltype(k_)::value;
    v[k1] = ex[(k1 * P + p) * 32 + lane];
  });
  reg::dft<R1, true>(v);
  group_sync(bar_id, P * 32);   // the exchange buffer is free again
}

template <int R, typename C> __device__ __forceinline__ void conj_all(C (&a)[R]) {
#pragma unroll
  for (int i = 0; i < R; ++i) a[i].y = -a[i].y;
}

// The same filter with less code, for the double-float type: each pair
// operation is 7-11 FP32 instructions, and the fully unrolled four_step (four
// codelets, called twice per fused kernel) overflows the instruction cache
// (measured: instruction-fetch stalls dominate).  Here the inverse DFTs are
// conj(DFT(conj(x))) and the forward and inverse halves run as rolled loops,
// so each codelet is emitted once.  Synchronises the whole CTA (bar 0).
template <int N, int P, typename C, typename T>
__device__ __forceinline__ void four_step_compact(C (&v)[N / P], C *ex, const C *tw,
                                                  const T *gain, int p, int lane) {
  constexpr int R1 = N / P;
#pragma unroll 1
  for (int phase = 0; phase < 2; ++phase) {
    if (phase == 1) {
      reg::static_for<0, R1>([&](auto k_) {
        constexpr int k1 = decltype(k_)::value;
        v[k1] = ex[(k1 * P + p) * 32 + lane];
      });
      conj_all(v);
    }
    reg::dft<R1, false>(v);
    if (phase == 1) {
      conj_all(v);
      break;
    }
    reg::static_for<0, R1>([&](auto k_) {
      constexpr int k1 = decltype(k_)::value;
      if (k1 > 0) v[k1] = cmul(v[k1], tw[p * k1]);
      ex[(k1 * P + p) * 32 + lane] = v[k1];
    });
    __syncthreads();
    for (int k1 = p; k1 < R1; k1 += P) {
      C u[P];
      reg::static_for<0, P>([&](auto q_) {
        constexpr int q = decltype(q_)::value;
        u[q] = ex[(k1 * P + q) * 32 + lane];
      });
#pragma unroll 1
      for (int dir = 0; dir < 2; ++dir) {
        reg::dft<P, false>(u);
        if (dir == 1) break;
        reg::static_for<0, P>([&](auto k2_) {
          constexpr int k2 = decltype(k2_)::value;
          const T g = gain[k1 + R1 * k2];
          u[k2].x *= g;
          u[k2].y *= g;
        });
        conj_all(u);
      }
      conj_all(u);
      reg::static_for<0, P>([&](auto q_) {
        constexpr int q = decltype(q_)::value;
        if (q > 0) u[q] = cmul(u[q], cconj(tw[q * k1]));
        ex[(k1 * P + q) * 32 + lane] = u[q];
      });
    }
    __syncthreads();
  }
  __syncthreads();   // the exchange buffer is free again
}

template <typename T> constexpr bool kCompactFilter = std::is_same<T, dfloat>::value;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

}  // namespace fcore
}  // namespace scft
