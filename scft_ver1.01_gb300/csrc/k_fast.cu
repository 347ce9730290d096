// Register-resident line filters, the fast propagator passes: per-axis
// passes (k_fast_line), x+y planes (k_xy_plane), fused step pairs (k_xyxy,
// k_zz, k_xx) and a pipelined column pass (k_col_pipe).  The real type is
// FP32, FP64 or the double-float pair (dfloat.cuh) where a kernel is
// templated on it; the plane kernels and the pipelined pass are FP32.
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
// Column passes (lines along y or z, stride s_n) load complex pairs straight
// from global memory: the 32 lanes of a warp read 64 consecutive x values
// (256 B in FP32, coalesced) per element.  The x pass stages a 64-row tile through shared
// memory (row pitch N+1 floats, conflict-free) and packs rows (l, l+32).
// The Boltzmann factor of the split step is applied on load (pre) and on
// store (post), so q makes one round trip per pass.
#include <type_traits>

#include "common.cuh"
#include "fft_reg.cuh"
#include "filter_core.cuh"
#include "kernels.h"

namespace scft {

namespace {

using namespace fcore;

// Offset of column c (of a column pass's tile row) in one instance's grid:
// the outer group blockIdx.y, or with flattened columns (ap.flat_nx) the row
// c / flat_nx.  Two-real pairs and 16-byte copies never straddle rows
// (flat_nx is a multiple of 4).
__device__ __forceinline__ long long col_off(const AxisPlan &ap, long long c) {
  if (ap.flat_nx) return (c / ap.flat_nx) * ap.s_outer + c % ap.flat_nx;
  return (long long)blockIdx.y * ap.s_outer + c;
}

// Shared memory of k_fast_line before its tables: the exchange buffer
// (N x 32 complex), or the 64-row staging tile (pitch N+1) of the x pass,
// for real type T (float or double).
template <typename T, int N, bool XP> __host__ __device__ constexpr size_t fast_core_smem() {
  return ((size_t)N * 32 * 2 * sizeof(T) > (XP ? (size_t)64 * (N + 1) * sizeof(T) : 0))
             ? (size_t)N * 32 * 2 * sizeof(T)
             : (((size_t)64 * (N + 1) * sizeof(T) + 15) / 16) * 16;
}


// Column passes keep the Boltzmann-factor tile of their output (N rows x 64
// reals) in shared memory after the twiddle/gain tables.  In double-float
// the tile would take 64 KB at N = 128 and leave room for one CTA (8 warps)
// per SM although the registers allow two; those kernels read the factor from
// global memory (an L2 hit) in their epilogue instead.  The FP64 kernels are
// register-bound at one CTA per SM, so they keep the prefetched tile.
template <typename T> constexpr bool kFactorTile = !std::is_same<T, dfloat>::value;

// Programmatic dependent launch for the register kernels of real type T.  The
// double-float kernels launch without it: their early-launched CTAs (two per
// SM, 71 KB each) wait resident for the predecessor and keep the other march
// chain's CTAs off those SMs (measured at 128^3: 21.46 ms per SCF iteration
// with PDL, 20.41 ms without; FP32 the other way: 4.32 against 4.47 ms).
template <typename T> constexpr bool kPdl = !std::is_same<T, dfloat>::value;
template <typename T, int N, bool XP> __host__ __device__ constexpr size_t fast_wtile_off() {
  return ((fast_core_smem<T, N, XP>() + (size_t)filter_table_reals<N>() * sizeof(T) + 15) / 16) *
         16;
}


template <typename T, int N, int P, bool XP>
__global__ void __launch_bounds__(P * 32) k_fast_line(AxisPlan ap, PassSet<T> ps) {
  using C = typename cplx<T>::type;
  constexpr int R1 = N / P;
  constexpr int NT = P * 32;
  constexpr int EPC = 16 / (int)sizeof(T);   // reals per 16-byte copy
  extern __shared__ __align__(128) unsigned char smem_raw[];
  C *ex = reinterpret_cast<C *>(smem_raw);
  const int lane = threadIdx.x & 31, p = threadIdx.x >> 5;
  // blockIdx.z = set * batch + instance
  const int set = (int)blockIdx.z >= ps.batch ? 1 : 0;
  long long b = (long long)blockIdx.z - (long long)set * ps.batch;
  const T *in = set ? ps.in[1] : ps.in[0];
  T *out = set ? ps.out[1] : ps.out[0];
  const T *pre = set ? ps.pre[1] : ps.pre[0];
  const T *post = set ? ps.post[1] : ps.post[0];
  const long long in_bs = set ? ps.in_bs[1] : ps.in_bs[0];
  const long long out_bs = set ? ps.out_bs[1] : ps.out_bs[0];
  const long long w_bs = ps.w_bs;
  const T *gain_n = reinterpret_cast<const T *>(ap.gain);
  if constexpr (std::is_same<T, float>::value) {
    if (ps.desc) {   // a batched pass: this line set's own buffers and gains
      const PassDesc d = ps.desc[blockIdx.z];
      in = d.in;
      out = d.out;
      pre = d.pre;
      post = d.post;
      gain_n = d.gain;
      b = 0;
    }
  }
  // The twiddle and gain tables go to shared memory first: they do not depend
  // on the previous pass, so this overlaps its tail, and the FFT stages then
  // read them with shared-memory broadcasts instead of dependent global loads.
  C *s_tw = reinterpret_cast<C *>(smem_raw + fast_core_smem<T, N, XP>());
  T *s_g = reinterpret_cast<T *>(s_tw + (kCompactFilter<T> ? N : 2 * N));
  if constexpr (kCompactFilter<T>)
    load_natural_tables<N>(s_tw, s_g, reinterpret_cast<const C *>(ap.twiddle), gain_n,
                           threadIdx.x, NT);
  else
    load_filter_tables<N, P>(s_tw, s_g, reinterpret_cast<const C *>(ap.twiddle), gain_n,
                             threadIdx.x, NT);
  // Column passes with a post factor: the factor's tile does not depend on
  // the previous pass either, so its cp.async copies are issued here too and
  // land while the lines are loaded and filtered (the epilogue then reads
  // shared memory instead of waiting on global loads).
  T *s_wt = reinterpret_cast<T *>(smem_raw + fast_wtile_off<T, N, XP>());
  if constexpr (!XP && kFactorTile<T>) {
    if (post) {
      constexpr int CPR = 64 / EPC;   // 16-byte copies per tile row of 64 reals
      const T *wt = post + b * w_bs;
      for (int c = threadIdx.x; c < N * CPR; c += NT) {
        const int row = c / CPR, part = c % CPR;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                         smem_addr(s_wt + row * 64 + part * EPC)),
                     "l"(wt + col_off(ap, (long long)blockIdx.x * 64 + part * EPC) +
                         (long long)row * ap.s_n)
                     : "memory");
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
    }
  }
  // the input slice is the previous pass's output
  pdl_wait();
  pdl_release();
  C v[R1];
  long long base;

  if constexpr (XP) {
    constexpr int PITCH = N + 1;
    T *stg = reinterpret_cast<T *>(smem_raw);
    base = (long long)blockIdx.x * 64 * N;  // 64 consecutive rows of N reals
    const T *src = in + b * in_bs + base;
    const T *wsrc = pre ? pre + b * w_bs + base : nullptr;
#pragma unroll
    for (int i = threadIdx.x; i < 64 * N; i += NT) {
      const int r = i / N, c = i % N;
      T x = ldg(src + i);
      if (wsrc) x *= ldg(wsrc + i);
      stg[r * PITCH + c] = x;
    }
    __syncthreads();
    reg::static_for<0, R1>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      const int n = p + P * j;
      v[j] = mkc<C, T>(stg[lane * PITCH + n], stg[(lane + 32) * PITCH + n]);
    });
    __syncthreads();
  } else {
    base = col_off(ap, (long long)blockIdx.x * 64 + 2 * lane);
    const T *src = in + b * in_bs + base;
    reg::static_for<0, R1>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      v[j] = ldg(reinterpret_cast<const C *>(src + (long long)(p + P * j) * ap.s_n));
    });
    if (pre) {
      const T *ws = pre + b * w_bs + base;
      reg::static_for<0, R1>([&](auto j_) {
        constexpr int j = decltype(j_)::value;
        const C w = ldg(reinterpret_cast<const C *>(ws + (long long)(p + P * j) * ap.s_n));
        v[j].x *= w.x;
        v[j].y *= w.y;
      });
    }
    __syncthreads();   // the shared tables are complete
  }

  if constexpr (kCompactFilter<T>) four_step_compact<N, P>(v, ex, s_tw, s_g, p, lane);
  else four_step<N, P>(v, ex, s_tw, s_g, p, lane, 0, []() {});

  if constexpr (XP) {
    constexpr int PITCH = N + 1;
    T *stg = reinterpret_cast<T *>(smem_raw);
    reg::static_for<0, R1>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      const int n = p + P * j;
      stg[lane * PITCH + n] = v[j].x;
      stg[(lane + 32) * PITCH + n] = v[j].y;
    });
    __syncthreads();
    T *dst = out + b * out_bs + base;
    const T *wdst = post ? post + b * w_bs + base : nullptr;
#pragma unroll 4
    for (int i = threadIdx.x; i < 64 * N; i += NT) {
      const int r = i / N, c = i % N;
      T x = stg[r * PITCH + c];
      if (wdst) x *= ldg(wdst + i);
      dst[i] = x;
    }
  } else {
    T *dst = out + b * out_bs + base;
    if (kFactorTile<T> && post) {
      asm volatile("cp.async.wait_all;" ::: "memory");
      __syncthreads();   // every thread's tile copies are visible
    }
    reg::static_for<0, R1>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      const long long off = (long long)(p + P * j) * ap.s_n;
      C r = v[j];
      if (post) {
        C w;
        if constexpr (kFactorTile<T>) w = reinterpret_cast<const C *>(s_wt)[(p + P * j) * 32 + lane];
        else w = ldg(reinterpret_cast<const C *>(post + b * w_bs + base + off));
        r.x *= w.x;
        r.y *= w.y;
      }
      *reinterpret_cast<C *>(dst + off) = r;
    });
  }
}

// ---- mbarrier / bulk-copy helpers (bounded waits) ------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
// 1-D bulk copy global -> shared (the TMA unit), completing on `bar`.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// Wait for phase `parity` of `bar`, for at most `limit` SM clocks (default
// ~1 s); false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity,
                                          long long limit = 2000000000LL) {
  const long long t0 = clock64();
  while (true) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > limit) return false;
  }
}

// Self-test of the bounded wait: an mbarrier that nothing ever arrives at is
// waited on for `limit` clocks; the timeout must set the error word and the
// kernel must return (nothing traps or hangs).
__global__ void k_wait_selftest(unsigned *err, long long limit) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (threadIdx.x == 0 && !mbar_wait(&bar, 0, limit)) atomicOr(err, 4u);
  __syncthreads();
}

// Persistent, pipelined column pass (lines along y or z).  Each CTA loops over
// tiles (set, instance, outer, 64-wide x-chunk); warp 0 stages the q rows of
// the next tiles into a two-slot shared-memory ring with cp.async.bulk
// (256 B per line element, completing on an mbarrier per slot) while all
// warps filter the current tile in registers.  W is read with plain loads
// issued before the slot wait.  Output is stored straight from registers.
template <int N, int P>
__global__ void __launch_bounds__(P * 32, N <= 128 ? 2 : 1)
    k_col_pipe(AxisPlan ap, PassSet<float> ps, unsigned *err) {
  constexpr int R1 = N / P;
  constexpr unsigned kTileBytes = N * 64 * 4;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float *slot[2] = {reinterpret_cast<float *>(smem_raw),
                    reinterpret_cast<float *>(smem_raw) + N * 64};
  float2 *ex = reinterpret_cast<float2 *>(smem_raw + 2 * kTileBytes);
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw + 3 * kTileBytes);
  float2 *tw = reinterpret_cast<float2 *>(smem_raw + 3 * kTileBytes + 16);
  float *gain = reinterpret_cast<float *>(tw + 2 * N);
  const int lane = threadIdx.x & 31, p = threadIdx.x >> 5;
  const int ntx = ap.n_real / 64;
  const long long T = (long long)ps.nset * ps.batch * ap.n_outer * ntx;
  load_filter_tables<N, P>(tw, gain, reinterpret_cast<const float2 *>(ap.twiddle),
                           reinterpret_cast<const float *>(ap.gain), threadIdx.x, P * 32);

  struct Tile {
    const float *in;
    float *out;
    const float *w;     // W at this tile (pre or post), or null
    bool pre;
  };
  auto tile_of = [&](long long t) {
    const int xt = (int)(t % ntx);
    long long r = t / ntx;
    const int outer = (int)(r % ap.n_outer);
    r /= ap.n_outer;
    const long long b = r % ps.batch;
    const int set = (int)(r / ps.batch);
    const long long off = (long long)outer * ap.s_outer + (long long)xt * 64;
    Tile tl;
    tl.in = (set ? ps.in[1] : ps.in[0]) + b * (set ? ps.in_bs[1] : ps.in_bs[0]) + off;
    tl.out = (set ? ps.out[1] : ps.out[0]) + b * (set ? ps.out_bs[1] : ps.out_bs[0]) + off;
    const float *pre = set ? ps.pre[1] : ps.pre[0];
    const float *post = set ? ps.post[1] : ps.post[0];
    tl.pre = pre != nullptr;
    tl.w = pre ? pre + b * ps.w_bs + off : (post ? post + b * ps.w_bs + off : nullptr);
    return tl;
  };
  // warp 0: stage tile t into slot s
  auto issue = [&](long long t, int s) {
    if (p != 0 || t >= T) return;
    const Tile tl = tile_of(t);
    if (lane == 0) mbar_expect_tx(&bar[s], kTileBytes);
    __syncwarp();
#pragma unroll
    for (int n = lane; n < N; n += 32)
      bulk_g2s(slot[s] + n * 64, tl.in + (long long)n * ap.s_n, 256, &bar[s]);
  };

  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  pdl_wait();      // inputs are the previous pass's output
  pdl_release();
  long long t = blockIdx.x;
  issue(t, 0);
  issue(t + gridDim.x, 1);
  for (int it = 0; t < T; ++it, t += gridDim.x) {
    const int s = it & 1;
    const unsigned parity = (it >> 1) & 1;
    const Tile tl = tile_of(t);
    float2 wv[R1];
    if (tl.w && tl.pre) {
      reg::static_for<0, R1>([&](auto j_) {
        constexpr int j = decltype(j_)::value;
        wv[j] = __ldg(reinterpret_cast<const float2 *>(tl.w + (long long)(p + P * j) * ap.s_n +
                                                        2 * lane));
      });
    }
    // block-uniform give-up: every thread leaves together, none is left at a barrier
    if (!__syncthreads_and(mbar_wait(&bar[s], parity) ? 1 : 0)) {
      if (threadIdx.x == 0) atomicOr(err, 1u);
      return;
    }
    float2 v[R1];
    reg::static_for<0, R1>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      v[j] = reinterpret_cast<const float2 *>(slot[s] + (p + P * j) * 64)[lane];
      if (tl.w && tl.pre) {
        v[j].x *= wv[j].x;
        v[j].y *= wv[j].y;
      }
    });
    four_step<N, P>(v, ex, tw, gain, p, lane, 0, [&]() {
      // every warp has read slot s: refill it with the tile after next
      if (p == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(t + 2LL * gridDim.x, s);
    });
    reg::static_for<0, R1>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      const long long off = (long long)(p + P * j) * ap.s_n + 2 * lane;
      float2 r = v[j];
      if (tl.w && !tl.pre) {
        const float2 w = __ldg(reinterpret_cast<const float2 *>(tl.w + off));
        r.x *= w.x;
        r.y *= w.y;
      }
      *reinterpret_cast<float2 *>(tl.out + off) = r;
    });
  }
}

template <int N, int P> size_t pipe_smem() {
  return (size_t)3 * N * 64 * 4 + 16 + (size_t)filter_table_reals<N>() * 4;
}

// ------------------------------------------------------------------------
// Fused x+y pass: one CTA per z-plane.  The plane (NY rows, pitch NX+1) sits
// in shared memory; the x pass filters its rows (lane l packs rows l+32r and
// l+32r+NY/2) and writes them back in place, then the y pass filters its
// columns (lane l packs columns 64r+l and 64r+l+32) and stores straight to
// global memory.  Saves one launch and one L2 round trip per contour step
// compared with separate x and y passes.
template <int NX, int NY> constexpr size_t xy_plane_bytes() {
  return (((size_t)NY * (NX + 1) * 4 + 127) / 128) * 128;
}
// G warp groups of 8 warps: group g takes rounds g, g+G, ... of each pass with
// its own exchange buffer and named barrier, so G groups keep G planes' worth
// of independent work in flight per plane.
template <int NX, int NY, int G> constexpr size_t xy_smem() {
  return xy_plane_bytes<NX, NY>() + (size_t)G * (NX > NY ? NX : NY) * 32 * 8 +
         (size_t)(filter_table_reals<NX>() + filter_table_reals<NY>()) * 4;
}

template <int NX, int NY, int G>
__global__ void __launch_bounds__(256 * G, G == 1 ? 2 : 1)
    k_xy_plane(AxisPlan apx, AxisPlan apy, PassSet<float> ps) {
  constexpr int P = 8, NT = 256 * G, PITCH = NX + 1;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float *plane = reinterpret_cast<float *>(smem_raw);
  const int grp = G == 1 ? 0 : (int)(threadIdx.x >> 8);
  float2 *ex0 = reinterpret_cast<float2 *>(smem_raw + xy_plane_bytes<NX, NY>());
  float2 *ex = ex0 + grp * (NX > NY ? NX : NY) * 32;
  float2 *twx = ex0 + G * (NX > NY ? NX : NY) * 32;
  float2 *twy = twx + 2 * NX;
  float *gx = reinterpret_cast<float *>(twy + 2 * NY);
  float *gy = gx + NX;
  const int lane = threadIdx.x & 31, p = (threadIdx.x >> 5) & 7;
  const int bar_id = G == 1 ? 0 : 1 + grp;
  const int set = (int)blockIdx.z >= ps.batch ? 1 : 0;
  const long long b = (long long)blockIdx.z - (long long)set * ps.batch;
  const long long base = (long long)blockIdx.x * NX * NY;
  const float *in = (set ? ps.in[1] : ps.in[0]) + b * (set ? ps.in_bs[1] : ps.in_bs[0]) + base;
  float *out = (set ? ps.out[1] : ps.out[0]) + b * (set ? ps.out_bs[1] : ps.out_bs[0]) + base;
  const float *pre = set ? ps.pre[1] : ps.pre[0];
  const float *post = set ? ps.post[1] : ps.post[0];
  if (pre) pre += b * ps.w_bs + base;
  if (post) post += b * ps.w_bs + base;
  const float *gxn = reinterpret_cast<const float *>(apx.gain);
  const float *gyn = reinterpret_cast<const float *>(apy.gain);
  if (ps.desc) {   // a batched pass: this plane set's own buffers and gains
    const PassDesc d = ps.desc[blockIdx.z];
    in = d.in + base;
    out = d.out + base;
    pre = d.pre ? d.pre + base : nullptr;
    post = d.post ? d.post + base : nullptr;
    gxn = d.gain;
    gyn = d.gain_y;
  }
  load_filter_tables<NX, P>(twx, gx, reinterpret_cast<const float2 *>(apx.twiddle), gxn,
                            threadIdx.x, NT);
  load_filter_tables<NY, P>(twy, gy, reinterpret_cast<const float2 *>(apy.twiddle), gyn,
                            threadIdx.x, NT);
  // The Boltzmann factor does not depend on the previous pass: its loads are
  // issued before the dependency wait and overlap that pass's tail.  Then
  // every load of the plane is in flight at once (NX*NY/NT per thread):
  // +4% at 128^3 over 8 in flight, measured; staging through cp.async was
  // slower.
  constexpr int PER = NX * NY / NT;
  float wr[PER];
#pragma unroll
  for (int k = 0; k < PER; ++k) wr[k] = pre ? __ldg(pre + threadIdx.x + k * NT) : 1.0f;
  pdl_wait();   // the plane is the previous pass's output
  pdl_release();
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const int i = threadIdx.x + k * NT;
    plane[(i / NX) * PITCH + (i % NX)] = __ldg(in + i) * wr[k];
  }
  __syncthreads();
  // x pass, NY/64 rounds of 32 complex rows
#pragma unroll 1
  for (int r = grp; r < NY / 64; r += G) {
    float2 v[NX / P];
    const int ra = r * 32 + lane, rb = ra + NY / 2;
    reg::static_for<0, NX / P>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      const int n = p + P * j;
      v[j] = make_float2(plane[ra * PITCH + n], plane[rb * PITCH + n]);
    });
    four_step<NX, P>(v, ex, twx, gx, p, lane, bar_id, []() {});
    reg::static_for<0, NX / P>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      const int n = p + P * j;
      plane[ra * PITCH + n] = v[j].x;
      plane[rb * PITCH + n] = v[j].y;
    });
  }
  __syncthreads();
  // y pass, NX/64 rounds of 32 complex columns, stored to global
#pragma unroll 1
  for (int r = grp; r < NX / 64; r += G) {
    float2 v[NY / P];
    const int ca = r * 64 + lane, cb = ca + 32;
    reg::static_for<0, NY / P>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      const int n = p + P * j;
      v[j] = make_float2(plane[n * PITCH + ca], plane[n * PITCH + cb]);
    });
    four_step<NY, P>(v, ex, twy, gy, p, lane, bar_id, []() {});
    reg::static_for<0, NY / P>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      const int n = p + P * j;
      float a = v[j].x, c = v[j].y;
      if (post) {
        a *= __ldg(post + n * NX + ca);
        c *= __ldg(post + n * NX + cb);
      }
      out[n * NX + ca] = a;
      out[n * NX + cb] = c;
    });
  }
}

// ------------------------------------------------------------------------
// Fused step pair on column lines (lines along z, or y when z is absent):
// finishes step s with the line filter and the post factor (stored to qout)
// and starts step s+1 with the factor again and the filter (stored to out).
// Geometry, tables and the cp.async factor tile as in the column branch of
// k_fast_line.
template <typename T, int N, int P>
__global__ void __launch_bounds__(P * 32) k_zz(AxisPlan ap, PassSet<T> ps) {
  using C = typename cplx<T>::type;
  constexpr int R1 = N / P;
  constexpr int NT = P * 32;
  constexpr int EPC = 16 / (int)sizeof(T);   // reals per 16-byte copy
  constexpr int CPR = 64 / EPC;              // copies per tile row of 64 reals
  extern __shared__ __align__(128) unsigned char smem_raw[];
  C *ex = reinterpret_cast<C *>(smem_raw);
  const int lane = threadIdx.x & 31, p = threadIdx.x >> 5;
  const int set = (int)blockIdx.z >= ps.batch ? 1 : 0;
  const long long b = (long long)blockIdx.z - (long long)set * ps.batch;
  const T *__restrict__ in = ps.in[set];
  T *__restrict__ out = ps.out[set];
  T *__restrict__ qo = ps.qout[set];
  const T *__restrict__ w = ps.post[set];
  C *s_tw = reinterpret_cast<C *>(smem_raw + fast_core_smem<T, N, false>());
  T *s_g = reinterpret_cast<T *>(s_tw + (kCompactFilter<T> ? N : 2 * N));
  if constexpr (kCompactFilter<T>)
    load_natural_tables<N>(s_tw, s_g, reinterpret_cast<const C *>(ap.twiddle),
                           reinterpret_cast<const T *>(ap.gain), threadIdx.x, NT);
  else
    load_filter_tables<N, P>(s_tw, s_g, reinterpret_cast<const C *>(ap.twiddle),
                             reinterpret_cast<const T *>(ap.gain), threadIdx.x, NT);
  T *s_wt = reinterpret_cast<T *>(smem_raw + fast_wtile_off<T, N, false>());
  const long long tile = (long long)blockIdx.y * ap.s_outer + (long long)blockIdx.x * 64;
  if constexpr (kFactorTile<T>) {
    const T *wt = w + b * ps.w_bs + tile;
    for (int c = threadIdx.x; c < N * CPR; c += NT) {
      const int row = c / CPR, part = c % CPR;
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                       smem_addr(s_wt + row * 64 + part * EPC)),
                   "l"(wt + (long long)row * ap.s_n + part * EPC)
                   : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  }
  pdl_wait();   // the input is the previous pass's output
  pdl_release();
  const long long base = tile + 2 * lane;
  C v[R1];
  {
    const T *src = in + b * ps.in_bs[set] + base;
    reg::static_for<0, R1>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      v[j] = ldg(reinterpret_cast<const C *>(src + (long long)(p + P * j) * ap.s_n));
    });
  }
  __syncthreads();   // the shared tables are complete
  auto finish_step = [&]() {
    if constexpr (kFactorTile<T>) {
      asm volatile("cp.async.wait_all;" ::: "memory");
      __syncthreads();   // every thread's tile copies are visible
    }
    T *dq = qo + b * ps.qout_bs[set] + base;
    const T *wg = w + b * ps.w_bs + base;
    reg::static_for<0, R1>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      C wv;
      if constexpr (kFactorTile<T>) wv = reinterpret_cast<const C *>(s_wt)[(p + P * j) * 32 + lane];
      else wv = ldg(reinterpret_cast<const C *>(wg + (long long)(p + P * j) * ap.s_n));
      C r = v[j];
      r.x *= wv.x;
      r.y *= wv.y;
      *reinterpret_cast<C *>(dq + (long long)(p + P * j) * ap.s_n) = r;
      v[j] = mkc<C, T>(r.x * wv.x, r.y * wv.y);
    });
  };
  if constexpr (kCompactFilter<T>) {
#pragma unroll 1
    for (int half = 0; half < 2; ++half) {
      four_step_compact<N, P>(v, ex, s_tw, s_g, p, lane);
      if (half == 1) break;
      finish_step();
    }
  } else {
    four_step<N, P>(v, ex, s_tw, s_g, p, lane, 0, []() {});
    finish_step();
    four_step<N, P>(v, ex, s_tw, s_g, p, lane, 0, []() {});
  }
  T *dst = out + b * ps.out_bs[set] + base;
  reg::static_for<0, R1>([&](auto j_) {
    constexpr int j = decltype(j_)::value;
    *reinterpret_cast<C *>(dst + (long long)(p + P * j) * ap.s_n) = v[j];
  });
}

// Fused step pair on x lines (rows contiguous, as the x branch of
// k_fast_line: 64 rows per CTA staged through shared memory, pitch N+1).
// The factor's tile (64 rows x N, contiguous in memory) is copied with
// cp.async before the dependency wait.
template <typename T, int N> constexpr size_t xx_wtile_off() {
  return fast_wtile_off<T, N, true>();
}
template <typename T, int N> constexpr size_t xx_smem() {
  return xx_wtile_off<T, N>() + (kFactorTile<T> ? (size_t)64 * N * sizeof(T) : 0);
}

template <typename T, int N, int P>
__global__ void __launch_bounds__(P * 32) k_xx(AxisPlan ap, PassSet<T> ps) {
  using C = typename cplx<T>::type;
  constexpr int R1 = N / P;
  constexpr int NT = P * 32;
  constexpr int PITCH = N + 1;
  constexpr int EPC = 16 / (int)sizeof(T);
  extern __shared__ __align__(128) unsigned char smem_raw[];
  C *ex = reinterpret_cast<C *>(smem_raw);   // aliases the staging tile
  T *stg = reinterpret_cast<T *>(smem_raw);
  const int lane = threadIdx.x & 31, p = threadIdx.x >> 5;
  const int set = (int)blockIdx.z >= ps.batch ? 1 : 0;
  const long long b = (long long)blockIdx.z - (long long)set * ps.batch;
  C *s_tw = reinterpret_cast<C *>(smem_raw + fast_core_smem<T, N, true>());
  T *s_g = reinterpret_cast<T *>(s_tw + (kCompactFilter<T> ? N : 2 * N));
  if constexpr (kCompactFilter<T>)
    load_natural_tables<N>(s_tw, s_g, reinterpret_cast<const C *>(ap.twiddle),
                           reinterpret_cast<const T *>(ap.gain), threadIdx.x, NT);
  else
    load_filter_tables<N, P>(s_tw, s_g, reinterpret_cast<const C *>(ap.twiddle),
                             reinterpret_cast<const T *>(ap.gain), threadIdx.x, NT);
  const long long base = (long long)blockIdx.x * 64 * N;   // 64 consecutive rows
  T *s_wt = reinterpret_cast<T *>(smem_raw + xx_wtile_off<T, N>());
  const T *wg = ps.post[set] + b * ps.w_bs + base;
  if constexpr (kFactorTile<T>) {
    const T *wt = wg;
    for (int c = threadIdx.x; c < 64 * N / EPC; c += NT)
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                       smem_addr(s_wt + EPC * c)),
                   "l"(wt + EPC * c)
                   : "memory");
    asm volatile("cp.async.commit_group;" ::: "memory");
  }
  pdl_wait();   // the rows are the previous pass's output
  pdl_release();
  const T *src = ps.in[set] + b * ps.in_bs[set] + base;
#pragma unroll
  for (int i = threadIdx.x; i < 64 * N; i += NT) stg[(i / N) * PITCH + (i % N)] = ldg(src + i);
  __syncthreads();
  C v[R1];
  auto rows_to_regs = [&]() {
    reg::static_for<0, R1>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      const int n = p + P * j;
      v[j] = mkc<C, T>(stg[lane * PITCH + n], stg[(lane + 32) * PITCH + n]);
    });
    __syncthreads();   // the staging tile is free for the exchange
  };
  auto regs_to_rows = [&]() {
    reg::static_for<0, R1>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      const int n = p + P * j;
      stg[lane * PITCH + n] = v[j].x;
      stg[(lane + 32) * PITCH + n] = v[j].y;
    });
    __syncthreads();
  };
  auto finish_step = [&]() {
    if constexpr (kFactorTile<T>) {
      asm volatile("cp.async.wait_all;" ::: "memory");
      __syncthreads();   // every thread's tile copies are visible
    }
    T *dq = ps.qout[set] + b * ps.qout_bs[set] + base;
#pragma unroll 4
    for (int i = threadIdx.x; i < 64 * N; i += NT) {
      const int o = (i / N) * PITCH + (i % N);
      T w;
      if constexpr (kFactorTile<T>) w = s_wt[i];
      else w = ldg(wg + i);
      const T x = stg[o] * w;
      dq[i] = x;
      stg[o] = x * w;
    }
    __syncthreads();
  };
  if constexpr (kCompactFilter<T>) {
#pragma unroll 1
    for (int half = 0; half < 2; ++half) {
      rows_to_regs();
      four_step_compact<N, P>(v, ex, s_tw, s_g, p, lane);
      regs_to_rows();
      if (half == 1) break;
      finish_step();
    }
  } else {
    rows_to_regs();
    four_step<N, P>(v, ex, s_tw, s_g, p, lane, 0, []() {});
    regs_to_rows();
    finish_step();
    rows_to_regs();
    four_step<N, P>(v, ex, s_tw, s_g, p, lane, 0, []() {});
    regs_to_rows();
  }
  T *dst = ps.out[set] + b * ps.out_bs[set] + base;
#pragma unroll 4
  for (int i = threadIdx.x; i < 64 * N; i += NT) dst[i] = stg[(i / N) * PITCH + (i % N)];
}

// Fused step pair on whole z-planes: x and y filters (finishing step s: the
// post factor, stored to qout), the factor again, then y and x filters of
// step s+1 (the filters commute), stored to out.  The plane and the factor's
// plane (cp.async, issued before the dependency wait) sit in shared memory.
template <int NX, int NY> constexpr size_t xyxy_wplane_off() {
  return xy_plane_bytes<NX, NY>();
}
template <int NX, int NY, int G> constexpr size_t xyxy_smem() {
  return xy_plane_bytes<NX, NY>() + (size_t)NX * NY * 4 +
         (size_t)G * (NX > NY ? NX : NY) * 32 * 8 +
         (size_t)(filter_table_reals<NX>() + filter_table_reals<NY>()) * 4;
}

template <int NX, int NY, int G>
__global__ void __launch_bounds__(256 * G, 1)
    k_xyxy(AxisPlan apx, AxisPlan apy, PassSet<float> ps) {
  constexpr int P = 8, NT = 256 * G, PITCH = NX + 1;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float *plane = reinterpret_cast<float *>(smem_raw);
  float *wplane = reinterpret_cast<float *>(smem_raw + xyxy_wplane_off<NX, NY>());
  const int grp = G == 1 ? 0 : (int)(threadIdx.x >> 8);
  float2 *ex0 = reinterpret_cast<float2 *>(smem_raw + xyxy_wplane_off<NX, NY>() +
                                           (size_t)NX * NY * 4);
  float2 *ex = ex0 + grp * (NX > NY ? NX : NY) * 32;
  float2 *twx = ex0 + G * (NX > NY ? NX : NY) * 32;
  float2 *twy = twx + 2 * NX;
  float *gx = reinterpret_cast<float *>(twy + 2 * NY);
  float *gy = gx + NX;
  const int lane = threadIdx.x & 31, p = (threadIdx.x >> 5) & 7;
  const int bar_id = G == 1 ? 0 : 1 + grp;
  const int set = (int)blockIdx.z >= ps.batch ? 1 : 0;
  const long long b = (long long)blockIdx.z - (long long)set * ps.batch;
  const long long base = (long long)blockIdx.x * NX * NY;
  const float *in = ps.in[set] + b * ps.in_bs[set] + base;
  float *out = ps.out[set] + b * ps.out_bs[set] + base;
  float *qo = ps.qout[set] + b * ps.qout_bs[set] + base;
  const float *w = ps.post[set] + b * ps.w_bs + base;
  load_filter_tables<NX, P>(twx, gx, reinterpret_cast<const float2 *>(apx.twiddle),
                            reinterpret_cast<const float *>(apx.gain), threadIdx.x, NT);
  load_filter_tables<NY, P>(twy, gy, reinterpret_cast<const float2 *>(apy.twiddle),
                            reinterpret_cast<const float *>(apy.gain), threadIdx.x, NT);
  for (int c = threadIdx.x; c < NX * NY / 4; c += NT)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(wplane + 4 * c)),
                 "l"(w + 4 * c)
                 : "memory");
  asm volatile("cp.async.commit_group;" ::: "memory");
  pdl_wait();   // the plane is the previous pass's output
  pdl_release();
  constexpr int PER = NX * NY / NT;
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const int i = threadIdx.x + k * NT;
    plane[(i / NX) * PITCH + (i % NX)] = __ldg(in + i);
  }
  __syncthreads();
  auto x_pass = [&]() {
#pragma unroll 1
    for (int r = grp; r < NY / 64; r += G) {
      float2 v[NX / P];
      const int ra = r * 32 + lane, rb = ra + NY / 2;
      reg::static_for<0, NX / P>([&](auto j_) {
        constexpr int j = decltype(j_)::value;
        const int n = p + P * j;
        v[j] = make_float2(plane[ra * PITCH + n], plane[rb * PITCH + n]);
      });
      four_step<NX, P>(v, ex, twx, gx, p, lane, bar_id, []() {});
      reg::static_for<0, NX / P>([&](auto j_) {
        constexpr int j = decltype(j_)::value;
        const int n = p + P * j;
        plane[ra * PITCH + n] = v[j].x;
        plane[rb * PITCH + n] = v[j].y;
      });
    }
  };
  x_pass();
  asm volatile("cp.async.wait_all;" ::: "memory");
  __syncthreads();   // rows filtered; the factor's plane is visible
  // y filter of step s, the factor (qout), the factor again, y filter of s+1
#pragma unroll 1
  for (int r = grp; r < NX / 64; r += G) {
    float2 v[NY / P];
    const int ca = r * 64 + lane, cb = ca + 32;
    reg::static_for<0, NY / P>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      const int n = p + P * j;
      v[j] = make_float2(plane[n * PITCH + ca], plane[n * PITCH + cb]);
    });
    four_step<NY, P>(v, ex, twy, gy, p, lane, bar_id, []() {});
    reg::static_for<0, NY / P>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      const int n = p + P * j;
      const float wa = wplane[n * NX + ca], wb = wplane[n * NX + cb];
      const float a = v[j].x * wa, c = v[j].y * wb;
      qo[n * NX + ca] = a;
      qo[n * NX + cb] = c;
      v[j] = make_float2(a * wa, c * wb);
    });
    four_step<NY, P>(v, ex, twy, gy, p, lane, bar_id, []() {});
    reg::static_for<0, NY / P>([&](auto j_) {
      constexpr int j = decltype(j_)::value;
      const int n = p + P * j;
      plane[n * PITCH + ca] = v[j].x;
      plane[n * PITCH + cb] = v[j].y;
    });
  }
  __syncthreads();
  x_pass();
  __syncthreads();
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const int i = threadIdx.x + k * NT;
    out[i] = plane[(i / NX) * PITCH + (i % NX)];
  }
}

template <typename T, int N, int P, bool XP> size_t fast_smem() {
  return XP ? fast_core_smem<T, N, XP>() + (size_t)filter_table_reals<N>() * sizeof(T)
            : fast_wtile_off<T, N, XP>() + (kFactorTile<T> ? (size_t)N * 64 * sizeof(T) : 0);
}

// Host-side shape checks of the tiled launches (the sanitizer substitute):
// the kernel's compile-time line length matches the plan, the 64-line tiles
// cover the lines exactly, and the grid fits CUDA's limits.  A failed check
// is an error status, never a launch.
template <typename T>
bool tiles_ok(const AxisPlan &ap, int n, bool outer_in_y, const PassSet<T> &ps) {
  const long long sets = (long long)ps.nset * ps.batch;
  return ap.n == n && ap.n_real > 0 && ap.n_real % 64 == 0 && sets >= 1 && sets <= 65535 &&
         (!outer_in_y || (ap.n_outer >= 1 && ap.n_outer <= 65535));
}
inline bool planes_ok(const AxisPlan &apx, const AxisPlan &apy, int nx, int ny,
                      const PassSet<float> &ps) {
  const long long sets = (long long)ps.nset * ps.batch;
  return apx.n == nx && apy.n == ny && apy.s_n == nx && apy.n_outer >= 1 && sets >= 1 &&
         sets <= 65535;
}

template <typename T, int N, int P, bool XP>
cudaError_t launch_one(const AxisPlan &ap, const PassSet<T> &ps, cudaStream_t st) {
  if (!tiles_ok(ap, N, !XP, ps)) return cudaErrorInvalidValue;
  dim3 grid(ap.n_real / 64, XP ? 1 : ap.n_outer, ps.nset * ps.batch);
  return launch_k(kPdl<T>, k_fast_line<T, N, P, XP>, grid, dim3(P * 32), fast_smem<T, N, P, XP>(), st,
                    ap, ps);
}

template <typename T, int N, int P, bool XP> cudaError_t prep_one() {
  return cudaFuncSetAttribute(k_fast_line<T, N, P, XP>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)fast_smem<T, N, P, XP>());
}

}  // namespace

bool fast_line_supported(const AxisPlan &ap, size_t real_bytes) {
  // FP64 lines stop at 128 points (256 would not fit the registers)
  if (ap.n != 32 && ap.n != 48 && ap.n != 64 && ap.n != 96 && ap.n != 128 &&
      !(ap.n == 256 && real_bytes == 4))
    return false;
  return ap.n_real % 64 == 0;
}

namespace {
constexpr int kMaxDev = 64;
int g_pipe_grid[kMaxDev][4];   // persistent grid size per device and N index (0: not set up)

template <int N, int P> cudaError_t prep_pipe(int dev, int idx) {
  cudaError_t e = cudaFuncSetAttribute(k_col_pipe<N, P>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)pipe_smem<N, P>());
  if (e != cudaSuccess) return e;
  int per_sm = 0, nsm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_col_pipe<N, P>, P * 32,
                                                    pipe_smem<N, P>());
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  g_pipe_grid[dev][idx] = (per_sm > 0 ? per_sm : 1) * nsm;
  return cudaSuccess;
}

template <int N, int P>
cudaError_t launch_pipe(const AxisPlan &ap, const PassSet<float> &ps, cudaStream_t st, int idx) {
  int dev = 0;
  cudaGetDevice(&dev);
  const long long T = (long long)ps.nset * ps.batch * ap.n_outer * (ap.n_real / 64);
  long long g = g_pipe_grid[dev][idx];
  if (g <= 0) return cudaErrorInitializationError;
  if (g > T) g = T;
  return launch_pdl(k_col_pipe<N, P>, dim3((unsigned)g), dim3(P * 32), pipe_smem<N, P>(), st, ap,
                    ps, ps.err);
}
// two warp groups when both passes have two rounds (128 x 128 planes)
// (one group of 256 threads at two CTAs per SM: -4% at 128^3, measured)
template <int NX, int NY> constexpr int xy_groups() { return (NX >= 128 && NY >= 128) ? 2 : 1; }

template <int NX, int NY> cudaError_t prep_xy() {
  constexpr int G = xy_groups<NX, NY>();
  return cudaFuncSetAttribute(k_xy_plane<NX, NY, G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)xy_smem<NX, NY, G>());
}
template <int NX, int NY>
cudaError_t launch_xy_t(const AxisPlan &apx, const AxisPlan &apy, const PassSet<float> &ps,
                        cudaStream_t st) {
  if (!planes_ok(apx, apy, NX, NY, ps)) return cudaErrorInvalidValue;
  constexpr int G = xy_groups<NX, NY>();
  dim3 grid(apy.n_outer, 1, ps.nset * ps.batch);   // one CTA per z-plane
  return launch_pdl(k_xy_plane<NX, NY, G>, grid, dim3(256 * G), xy_smem<NX, NY, G>(), st, apx,
                    apy, ps);
}
template <int NX, int NY> cudaError_t prep_xyxy() {
  constexpr int G = xy_groups<NX, NY>();
  return cudaFuncSetAttribute(k_xyxy<NX, NY, G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)xyxy_smem<NX, NY, G>());
}
template <int NX, int NY>
cudaError_t launch_xyxy_t(const AxisPlan &apx, const AxisPlan &apy, const PassSet<float> &ps,
                          cudaStream_t st) {
  if (!planes_ok(apx, apy, NX, NY, ps)) return cudaErrorInvalidValue;
  constexpr int G = xy_groups<NX, NY>();
  dim3 grid(apy.n_outer, 1, ps.nset * ps.batch);   // one CTA per z-plane
  return launch_pdl(k_xyxy<NX, NY, G>, grid, dim3(256 * G), xyxy_smem<NX, NY, G>(), st, apx,
                    apy, ps);
}
template <typename T, int N, int P> cudaError_t prep_xx() {
  return cudaFuncSetAttribute(k_xx<T, N, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)xx_smem<T, N>());
}
template <typename T, int N, int P>
cudaError_t launch_xx_t(const AxisPlan &ap, const PassSet<T> &ps, cudaStream_t st) {
  if (!tiles_ok(ap, N, false, ps)) return cudaErrorInvalidValue;
  dim3 grid(ap.n_real / 64, 1, ps.nset * ps.batch);
  return launch_k(kPdl<T>, k_xx<T, N, P>, grid, dim3(P * 32), xx_smem<T, N>(), st, ap, ps);
}
template <typename T, int N, int P> cudaError_t prep_zz() {
  return cudaFuncSetAttribute(k_zz<T, N, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)fast_smem<T, N, P, false>());
}
template <typename T, int N, int P>
cudaError_t launch_zz_t(const AxisPlan &ap, const PassSet<T> &ps, cudaStream_t st) {
  if (!tiles_ok(ap, N, true, ps)) return cudaErrorInvalidValue;
  dim3 grid(ap.n_real / 64, ap.n_outer, ps.nset * ps.batch);
  return launch_k(kPdl<T>, k_zz<T, N, P>, grid, dim3(P * 32), fast_smem<T, N, P, false>(), st, ap,
                    ps);
}
// 16-byte cp.async tiles and two-real lines: refuse misaligned buffers
template <typename T> bool fused_aligned(const PassSet<T> &ps) {
  for (int k = 0; k < ps.nset; ++k)
    if ((reinterpret_cast<uintptr_t>(ps.post[k]) | reinterpret_cast<uintptr_t>(ps.in[k]) |
         reinterpret_cast<uintptr_t>(ps.out[k]) | reinterpret_cast<uintptr_t>(ps.qout[k])) & 15 ||
        !ps.post[k] || !ps.qout[k])
      return false;
  return true;
}
}  // namespace

cudaError_t launch_xx(const AxisPlan &ap, const PassSet<float> &ps, cudaStream_t st) {
  if (ps.nset < 1 || ps.nset > kMaxSet || !ap.n_fast) return cudaErrorInvalidValue;
  if (!fused_aligned(ps)) return cudaErrorMisalignedAddress;
  switch (ap.n) {
    case 32: return launch_xx_t<float, 32, 4>(ap, ps, st);
    case 48: return launch_xx_t<float, 48, 8>(ap, ps, st);
    case 64: return launch_xx_t<float, 64, 8>(ap, ps, st);
    case 96: return launch_xx_t<float, 96, 8>(ap, ps, st);
    case 128: return launch_xx_t<float, 128, 8>(ap, ps, st);
    case 256: return launch_xx_t<float, 256, 16>(ap, ps, st);
    default: return cudaErrorInvalidValue;
  }
}
// 8-byte reals (FP64 and double-float): lines up to 128 points fit the registers
namespace {
template <typename T>
cudaError_t launch_xx_wide(const AxisPlan &ap, const PassSet<T> &ps, cudaStream_t st) {
  if (ps.nset < 1 || ps.nset > kMaxSet || !ap.n_fast) return cudaErrorInvalidValue;
  if (!fused_aligned(ps)) return cudaErrorMisalignedAddress;
  switch (ap.n) {
    case 32: return launch_xx_t<T, 32, 4>(ap, ps, st);
    case 64: return launch_xx_t<T, 64, 8>(ap, ps, st);
    case 128: return launch_xx_t<T, 128, 8>(ap, ps, st);
    default: break;
  }
  if constexpr (std::is_same<T, double>::value) {
    if (ap.n == 48) return launch_xx_t<T, 48, 8>(ap, ps, st);
    if (ap.n == 96) return launch_xx_t<T, 96, 8>(ap, ps, st);
  }
  return cudaErrorInvalidValue;
}
template <typename T>
cudaError_t launch_zz_wide(const AxisPlan &ap, const PassSet<T> &ps, cudaStream_t st) {
  if (ps.nset < 1 || ps.nset > kMaxSet || ap.n_fast) return cudaErrorInvalidValue;
  if (!fused_aligned(ps)) return cudaErrorMisalignedAddress;
  switch (ap.n) {
    case 32: return launch_zz_t<T, 32, 4>(ap, ps, st);
    case 64: return launch_zz_t<T, 64, 8>(ap, ps, st);
    case 128: return launch_zz_t<T, 128, 8>(ap, ps, st);
    default: break;
  }
  if constexpr (std::is_same<T, double>::value) {
    if (ap.n == 48) return launch_zz_t<T, 48, 8>(ap, ps, st);
    if (ap.n == 96) return launch_zz_t<T, 96, 8>(ap, ps, st);
  }
  return cudaErrorInvalidValue;
}
template <typename T>
cudaError_t launch_fast_line_wide(const AxisPlan &ap, const PassSet<T> &ps, cudaStream_t st) {
  if (ps.nset < 1 || ps.nset > kMaxSet) return cudaErrorInvalidValue;
  for (int k = 0; k < ps.nset; ++k)
    if ((reinterpret_cast<uintptr_t>(ps.post[k]) | reinterpret_cast<uintptr_t>(ps.pre[k]) |
         reinterpret_cast<uintptr_t>(ps.in[k]) | reinterpret_cast<uintptr_t>(ps.out[k])) & 15)
      return cudaErrorMisalignedAddress;
  const bool xp = ap.n_fast != 0;
  switch (ap.n) {
    case 32:
      return xp ? launch_one<T, 32, 4, true>(ap, ps, st) : launch_one<T, 32, 4, false>(ap, ps, st);
    case 64:
      return xp ? launch_one<T, 64, 8, true>(ap, ps, st) : launch_one<T, 64, 8, false>(ap, ps, st);
    case 128:
      return xp ? launch_one<T, 128, 8, true>(ap, ps, st)
                : launch_one<T, 128, 8, false>(ap, ps, st);
    default: break;
  }
  if constexpr (std::is_same<T, double>::value) {
    if (ap.n == 48)
      return xp ? launch_one<T, 48, 8, true>(ap, ps, st) : launch_one<T, 48, 8, false>(ap, ps, st);
    if (ap.n == 96)
      return xp ? launch_one<T, 96, 8, true>(ap, ps, st) : launch_one<T, 96, 8, false>(ap, ps, st);
  }
  return cudaErrorInvalidValue;
}
}  // namespace

cudaError_t launch_xx(const AxisPlan &ap, const PassSet<double> &ps, cudaStream_t st) {
  return launch_xx_wide(ap, ps, st);
}
cudaError_t launch_xx(const AxisPlan &ap, const PassSet<dfloat> &ps, cudaStream_t st) {
  return launch_xx_wide(ap, ps, st);
}

cudaError_t launch_wait_selftest(unsigned *err, long long limit, cudaStream_t st) {
  k_wait_selftest<<<1, 32, 0, st>>>(err, limit);
  return cudaGetLastError();
}

cudaError_t launch_zz(const AxisPlan &ap, const PassSet<float> &ps, cudaStream_t st) {
  if (ps.nset < 1 || ps.nset > kMaxSet || ap.n_fast) return cudaErrorInvalidValue;
  if (!fused_aligned(ps)) return cudaErrorMisalignedAddress;
  switch (ap.n) {
    case 32: return launch_zz_t<float, 32, 4>(ap, ps, st);
    case 48: return launch_zz_t<float, 48, 8>(ap, ps, st);
    case 64: return launch_zz_t<float, 64, 8>(ap, ps, st);
    case 96: return launch_zz_t<float, 96, 8>(ap, ps, st);
    case 128: return launch_zz_t<float, 128, 8>(ap, ps, st);
    case 256: return launch_zz_t<float, 256, 16>(ap, ps, st);
    default: return cudaErrorInvalidValue;
  }
}
cudaError_t launch_zz(const AxisPlan &ap, const PassSet<double> &ps, cudaStream_t st) {
  return launch_zz_wide(ap, ps, st);
}
cudaError_t launch_zz(const AxisPlan &ap, const PassSet<dfloat> &ps, cudaStream_t st) {
  return launch_zz_wide(ap, ps, st);
}

cudaError_t launch_xyxy(const AxisPlan &apx, const AxisPlan &apy, const PassSet<float> &ps,
                        cudaStream_t st) {
  if (ps.nset < 1 || ps.nset > kMaxSet) return cudaErrorInvalidValue;
  if (!fused_aligned(ps)) return cudaErrorMisalignedAddress;
  if (apx.n == 128 && apy.n == 128) return launch_xyxy_t<128, 128>(apx, apy, ps, st);
  if (apx.n == 64 && apy.n == 64) return launch_xyxy_t<64, 64>(apx, apy, ps, st);
  if (apx.n == 128 && apy.n == 64) return launch_xyxy_t<128, 64>(apx, apy, ps, st);
  if (apx.n == 64 && apy.n == 128) return launch_xyxy_t<64, 128>(apx, apy, ps, st);
  if (plane256_fusable(apx, apy)) return launch_xyxy256(apx, apy, ps, st);
  return cudaErrorInvalidValue;
}

bool xy_fusable(const AxisPlan &apx, const AxisPlan &apy) {
  if (plane256_fusable(apx, apy)) return true;
  return apx.n_fast && !apy.n_fast && (apx.n == 64 || apx.n == 128) &&
         (apy.n == 64 || apy.n == 128) && apy.s_n == apx.n && !apy.flat_nx;
}

cudaError_t launch_xy(const AxisPlan &apx, const AxisPlan &apy, const PassSet<float> &ps,
                      cudaStream_t st) {
  if (ps.nset < 1 || ps.nset > kMaxSet) return cudaErrorInvalidValue;
  if (apx.n == 128 && apy.n == 128) return launch_xy_t<128, 128>(apx, apy, ps, st);
  if (apx.n == 64 && apy.n == 64) return launch_xy_t<64, 64>(apx, apy, ps, st);
  if (apx.n == 128 && apy.n == 64) return launch_xy_t<128, 64>(apx, apy, ps, st);
  if (apx.n == 64 && apy.n == 128) return launch_xy_t<64, 128>(apx, apy, ps, st);
  if (plane256_fusable(apx, apy)) return launch_xy256(apx, apy, ps, st);
  return cudaErrorInvalidValue;
}

cudaError_t fast_line_prepare() {
  cudaError_t e = cudaSuccess;
#define PREP(T, N, P)                                              \
  if ((e = prep_one<T, N, P, false>()) != cudaSuccess) return e;  \
  if ((e = prep_one<T, N, P, true>()) != cudaSuccess) return e;
  PREP(float, 32, 4)
  PREP(float, 64, 8)
  PREP(float, 128, 8)
  PREP(float, 256, 16)
  PREP(float, 48, 8)
  PREP(float, 96, 8)
  PREP(double, 48, 8)
  PREP(double, 96, 8)
  PREP(double, 32, 4)
  PREP(double, 64, 8)
  PREP(double, 128, 8)
  PREP(dfloat, 32, 4)
  PREP(dfloat, 64, 8)
  PREP(dfloat, 128, 8)
#undef PREP
  int dev = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
  if ((e = prep_pipe<32, 4>(dev, 0)) != cudaSuccess) return e;
  if ((e = prep_pipe<64, 8>(dev, 1)) != cudaSuccess) return e;
  if ((e = prep_pipe<128, 8>(dev, 2)) != cudaSuccess) return e;
  if ((e = prep_pipe<256, 16>(dev, 3)) != cudaSuccess) return e;
  if ((e = prep_xy<128, 128>()) != cudaSuccess) return e;
  if ((e = prep_xy<64, 64>()) != cudaSuccess) return e;
  if ((e = prep_xy<128, 64>()) != cudaSuccess) return e;
  if ((e = prep_xy<64, 128>()) != cudaSuccess) return e;
  if ((e = prep_xyxy<128, 128>()) != cudaSuccess) return e;
  if ((e = prep_xyxy<64, 64>()) != cudaSuccess) return e;
  if ((e = prep_xyxy<128, 64>()) != cudaSuccess) return e;
  if ((e = prep_xyxy<64, 128>()) != cudaSuccess) return e;
  if ((e = plane256_prepare()) != cudaSuccess) return e;
#define PREP_FUSED(T, N, P)                                          \
  if ((e = prep_xx<T, N, P>()) != cudaSuccess) return e;            \
  if ((e = prep_zz<T, N, P>()) != cudaSuccess) return e;
  PREP_FUSED(float, 32, 4)
  PREP_FUSED(float, 64, 8)
  PREP_FUSED(float, 128, 8)
  PREP_FUSED(float, 256, 16)
  PREP_FUSED(float, 48, 8)
  PREP_FUSED(float, 96, 8)
  PREP_FUSED(double, 48, 8)
  PREP_FUSED(double, 96, 8)
  PREP_FUSED(double, 32, 4)
  PREP_FUSED(double, 64, 8)
  PREP_FUSED(double, 128, 8)
  PREP_FUSED(dfloat, 32, 4)
  PREP_FUSED(dfloat, 64, 8)
  PREP_FUSED(dfloat, 128, 8)
#undef PREP_FUSED
  return e;
}

cudaError_t launch_fast_line(const AxisPlan &ap, const PassSet<float> &ps, cudaStream_t st) {
  if (ps.nset < 1 || ps.nset > kMaxSet) return cudaErrorInvalidValue;
  // column passes copy their post-factor tile with 16-byte cp.async and move
  // lines as float2: refuse misaligned buffers instead of faulting
  for (int k = 0; k < ps.nset; ++k)
    if ((reinterpret_cast<uintptr_t>(ps.post[k]) | reinterpret_cast<uintptr_t>(ps.pre[k]) |
         reinterpret_cast<uintptr_t>(ps.in[k]) | reinterpret_cast<uintptr_t>(ps.out[k])) & 15)
      return cudaErrorMisalignedAddress;
  const bool xp = ap.n_fast != 0;
  // column passes: the persistent pipelined kernel when the caller supplied
  // an error word for its bounded waits
  if (!xp && ps.err && !ap.flat_nx) {
    switch (ap.n) {
      case 32: return launch_pipe<32, 4>(ap, ps, st, 0);
      case 64: return launch_pipe<64, 8>(ap, ps, st, 1);
      case 128: return launch_pipe<128, 8>(ap, ps, st, 2);
      case 256: return launch_pipe<256, 16>(ap, ps, st, 3);
      default: break;
    }
  }
  switch (ap.n) {
    case 32:
      return xp ? launch_one<float, 32, 4, true>(ap, ps, st)
                : launch_one<float, 32, 4, false>(ap, ps, st);
    case 64:
      return xp ? launch_one<float, 64, 8, true>(ap, ps, st)
                : launch_one<float, 64, 8, false>(ap, ps, st);
    case 128:
      return xp ? launch_one<float, 128, 8, true>(ap, ps, st)
                : launch_one<float, 128, 8, false>(ap, ps, st);
    case 256:
      return xp ? launch_one<float, 256, 16, true>(ap, ps, st)
                : launch_one<float, 256, 16, false>(ap, ps, st);
    case 48:
      return xp ? launch_one<float, 48, 8, true>(ap, ps, st)
                : launch_one<float, 48, 8, false>(ap, ps, st);
    case 96:
      return xp ? launch_one<float, 96, 8, true>(ap, ps, st)
                : launch_one<float, 96, 8, false>(ap, ps, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_fast_line(const AxisPlan &ap, const PassSet<double> &ps, cudaStream_t st) {
  return launch_fast_line_wide(ap, ps, st);
}
cudaError_t launch_fast_line(const AxisPlan &ap, const PassSet<dfloat> &ps, cudaStream_t st) {
  return launch_fast_line_wide(ap, ps, st);
}

}  // namespace scft
