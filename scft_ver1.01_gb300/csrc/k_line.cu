// Generic per-axis line filter: the correctness backbone of the propagator
// step (both precisions, any line length whose prime factors are <= 61).
//
// One propagator split step of the reference (sovDifFft, cuda_scft.cu:467-491:
// initilize_in_go -> cufftExecD2Z -> sufaceField_go -> cufftExecZ2D ->
// in_to_g_go) is  q_s = W . IFFT3[ G . FFT3[ W . q_{s-1} ] ] / M  with the
// reference's Gaussian table G = exp(-ds0*(kx^2+ky^2+kz^2))
// (init_cuda.cu:420-428).  G is a product of per-axis factors, so the 3D
// operator factorizes exactly into three 1D operators, one per axis; each is
// applied here to all lines along its axis: forward DFT, multiply by the real
// even gain g[k] = G_axis[k]/N, inverse DFT.  The inverse is computed as
// conj(DFT(conj(.))) so only a forward Stockham transform is needed.
//
// Tile: tl complex lines (2*tl real lines) of one outer group live in shared
// memory as two ping-pong buffers; each Stockham stage of radix p reads one
// buffer and writes the other (autosort, natural order in and out).
#include <type_traits>

#include "common.cuh"
#include "kernels.h"

namespace scft {

namespace {

template <typename R> struct K;
template <> struct K<float> {
  static __device__ __forceinline__ float s3() { return 0.866025403784438647f; }
  static __device__ __forceinline__ float c5a() { return 0.309016994374947424f; }   // cos(2pi/5)
  static __device__ __forceinline__ float c5b() { return -0.809016994374947424f; }  // cos(4pi/5)
  static __device__ __forceinline__ float s5a() { return 0.951056516295153572f; }   // sin(2pi/5)
  static __device__ __forceinline__ float s5b() { return 0.587785252292473129f; }   // sin(4pi/5)
};
template <> struct K<double> {
  static __device__ __forceinline__ double s3() { return 0.866025403784438647; }
  static __device__ __forceinline__ double c5a() { return 0.309016994374947424; }
  static __device__ __forceinline__ double c5b() { return -0.809016994374947424; }
  static __device__ __forceinline__ double s5a() { return 0.951056516295153572; }
  static __device__ __forceinline__ double s5b() { return 0.587785252292473129; }
};

// Forward DFT butterflies, X[k] = sum_r v[r] exp(-2 pi i r k / p).
template <typename R, typename C> __device__ __forceinline__ void dft2(C *v) {
  C a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}
template <typename R, typename C> __device__ __forceinline__ void dft3(C *v) {
  C a = v[0], b = v[1], c = v[2];
  C s = cadd(b, c), d = csub(b, c);
  v[0] = cadd(a, s);
  C m = mkc<C, R>(a.x - R(0.5) * s.x, a.y - R(0.5) * s.y);
  // -i*sin(2pi/3)*d
  C t = mkc<C, R>(K<R>::s3() * d.y, -K<R>::s3() * d.x);
  v[1] = cadd(m, t);
  v[2] = csub(m, t);
}
template <typename R, typename C> __device__ __forceinline__ void dft4(C *v) {
  C a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
  C c = cadd(v[1], v[3]), d = cmul_mi(csub(v[1], v[3]));
  v[0] = cadd(a, c);
  v[2] = csub(a, c);
  v[1] = cadd(b, d);
  v[3] = csub(b, d);
}
template <typename R, typename C> __device__ __forceinline__ void dft5(C *v) {
  C a = v[0];
  C s1 = cadd(v[1], v[4]), d1 = csub(v[1], v[4]);
  C s2 = cadd(v[2], v[3]), d2 = csub(v[2], v[3]);
  v[0] = cadd(a, cadd(s1, s2));
  C m1 = mkc<C, R>(a.x + K<R>::c5a() * s1.x + K<R>::c5b() * s2.x,
                   a.y + K<R>::c5a() * s1.y + K<R>::c5b() * s2.y);
  C m2 = mkc<C, R>(a.x + K<R>::c5b() * s1.x + K<R>::c5a() * s2.x,
                   a.y + K<R>::c5b() * s1.y + K<R>::c5a() * s2.y);
  // -i*(sa*d1 + sb*d2) and -i*(sb*d1 - sa*d2)
  R t1x = K<R>::s5a() * d1.x + K<R>::s5b() * d2.x, t1y = K<R>::s5a() * d1.y + K<R>::s5b() * d2.y;
  R t2x = K<R>::s5b() * d1.x - K<R>::s5a() * d2.x, t2y = K<R>::s5b() * d1.y - K<R>::s5a() * d2.y;
  v[1] = mkc<C, R>(m1.x + t1y, m1.y - t1x);
  v[4] = mkc<C, R>(m1.x - t1y, m1.y + t1x);
  v[2] = mkc<C, R>(m2.x + t2y, m2.y - t2x);
  v[3] = mkc<C, R>(m2.x - t2y, m2.y + t2x);
}

// One Stockham stage of radix P (compile-time) for all tile lines.
template <typename R, int P>
__device__ __forceinline__ void stage_fixed(const typename cplx<R>::type *src,
                                            typename cplx<R>::type *dst, int n, int ns,
                                            int tl, const typename cplx<R>::type *tw) {
  typedef typename cplx<R>::type C;
  const int nb = n / P;          // butterflies per line
  const int tstep = n / (ns * P);
  for (int idx = threadIdx.x; idx < tl * nb; idx += blockDim.x) {
    const int t = idx / nb, j = idx - t * nb;
    const C *s = src + t * n;
    C v[P];
    const int k = j % ns;
#pragma unroll
    for (int r = 0; r < P; ++r) v[r] = s[j + r * nb];
#pragma unroll
    for (int r = 1; r < P; ++r) {
      v[r] = cmul(v[r], tw[k * r * tstep]);  // k*r*tstep < n
    }
    if (P == 2) dft2<R>(v);
    else if (P == 3) dft3<R>(v);
    else if (P == 4) dft4<R>(v);
    else if (P == 5) dft5<R>(v);
    const int d0 = (j / ns) * ns * P + k;
    C *d = dst + t * n;
#pragma unroll
    for (int r = 0; r < P; ++r) d[d0 + r * ns] = v[r];
  }
}

// Generic radix (prime p <= 61): O(p^2) DFT through the twiddle table.
template <typename R>
__device__ void stage_generic(const typename cplx<R>::type *src, typename cplx<R>::type *dst,
                              int n, int ns, int p, int tl, const typename cplx<R>::type *tw) {
  typedef typename cplx<R>::type C;
  const int nb = n / p;
  const int tstep = n / (ns * p);
  const int pstep = n / p;
  for (int idx = threadIdx.x; idx < tl * nb; idx += blockDim.x) {
    const int t = idx / nb, j = idx - t * nb;
    const C *s = src + t * n;
    const int k = j % ns;
    C v[61];
    for (int r = 0; r < p; ++r) {
      C x = s[j + r * nb];
      v[r] = cmul(x, tw[k * r * tstep]);
    }
    const int d0 = (j / ns) * ns * p + k;
    C *d = dst + t * n;
    for (int q = 0; q < p; ++q) {
      C acc = mkc<C, R>(R(0), R(0));
      for (int r = 0; r < p; ++r) acc = cadd(acc, cmul(v[r], tw[((r * q) % p) * pstep]));
      d[d0 + q * ns] = acc;
    }
  }
}

template <typename R>
__device__ __forceinline__ typename cplx<R>::type *fft_forward(typename cplx<R>::type *a,
                                                               typename cplx<R>::type *b,
                                                               const AxisPlan &ap, int tl,
                                                               const typename cplx<R>::type *tw) {
  typename cplx<R>::type *src = a, *dst = b;
  int ns = 1;
  for (int f = 0; f < ap.nfac; ++f) {
    const int p = ap.fac[f];
    __syncthreads();
    switch (p) {
      case 2: stage_fixed<R, 2>(src, dst, ap.n, ns, tl, tw); break;
      case 3: stage_fixed<R, 3>(src, dst, ap.n, ns, tl, tw); break;
      case 4: stage_fixed<R, 4>(src, dst, ap.n, ns, tl, tw); break;
      case 5: stage_fixed<R, 5>(src, dst, ap.n, ns, tl, tw); break;
      default: stage_generic<R>(src, dst, ap.n, ns, p, tl, tw); break;
    }
    ns *= p;
    typename cplx<R>::type *t = src; src = dst; dst = t;
  }
  __syncthreads();
  return src;  // holds the result
}

template <typename R>
__global__ void __launch_bounds__(256) k_line_filter(AxisPlan ap, const R *__restrict__ in,
                                                     long long in_bs, R *__restrict__ out,
                                                     long long out_bs, const R *__restrict__ pre,
                                                     const R *__restrict__ post, long long w_bs,
                                                     const PassDesc *desc) {
  typedef typename cplx<R>::type C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = ap.n;
  const int n_pairs = (ap.n_real + 1) >> 1;
  const int c0 = blockIdx.x * ap.tl;
  const int tl = min(ap.tl, n_pairs - c0);
  const int outer = blockIdx.y;
  const int b = blockIdx.z;
  C *buf0 = reinterpret_cast<C *>(smem_raw);
  C *buf1 = buf0 + (size_t)ap.tl * n;
  R *rb0 = reinterpret_cast<R *>(buf0);
  const C *tw = reinterpret_cast<const C *>(ap.twiddle);
  const R *gain = reinterpret_cast<const R *>(ap.gain);
  pdl_wait();      // the input slice is the previous pass's output
  pdl_release();

  const long long base = (long long)outer * ap.s_outer;
  const R *inb = in + (long long)b * in_bs + base;
  R *outb = out + (long long)b * out_bs + base;
  const R *preb = pre ? pre + (long long)b * w_bs + base : nullptr;
  const R *postb = post ? post + (long long)b * w_bs + base : nullptr;
  if constexpr (std::is_same<R, float>::value) {
    if (desc) {   // a batched pass: this line set's own buffers and gains
      const PassDesc d = desc[b];
      inb = d.in + base;
      outb = d.out + base;
      preb = d.pre ? d.pre + base : nullptr;
      postb = d.post ? d.post + base : nullptr;
      gain = d.gain;
    }
  }

  // ---- load (two real lines -> one complex line)
  const int total = tl * 2 * n;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    int nn, h, t;
    if (ap.n_fast) { nn = idx % n; const int rem = idx / n; h = rem & 1; t = rem >> 1; }
    else { h = idx & 1; const int rem = idx >> 1; t = rem % tl; nn = rem / tl; }
    const int r = 2 * (c0 + t) + h;
    R v = R(0);
    if (r < ap.n_real) {
      const long long off = (long long)r * ap.s_pair + (long long)nn * ap.s_n;
      v = inb[off];
      if (preb) v *= preb[off];
    }
    rb0[2 * (t * n + nn) + h] = v;
  }

  // ---- forward DFT of every line
  C *res = fft_forward<R>(buf0, buf1, ap, tl, tw);
  // ---- multiply by the gain and conjugate (inverse = conj(DFT(conj(.))))
  for (int idx = threadIdx.x; idx < tl * n; idx += blockDim.x) {
    const int k = idx % n;
    C v = res[idx];
    const R g = gain[k];
    v.x *= g;
    v.y *= -g;
    res[idx] = v;
  }
  C *other = (res == buf0) ? buf1 : buf0;
  res = fft_forward<R>(res, other, ap, tl, tw);
  const R *rres = reinterpret_cast<const R *>(res);

  // ---- store (real part -> line 2c, -imag -> line 2c+1)
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    int nn, h, t;
    if (ap.n_fast) { nn = idx % n; const int rem = idx / n; h = rem & 1; t = rem >> 1; }
    else { h = idx & 1; const int rem = idx >> 1; t = rem % tl; nn = rem / tl; }
    const int r = 2 * (c0 + t) + h;
    if (r < ap.n_real) {
      const long long off = (long long)r * ap.s_pair + (long long)nn * ap.s_n;
      R v = rres[2 * (t * n + nn) + h];
      if (h) v = -v;
      if (postb) v *= postb[off];
      outb[off] = v;
    }
  }
}

}  // namespace

size_t line_filter_smem_bytes(const AxisPlan &ap, size_t real_bytes) {
  return 2 * (size_t)ap.tl * ap.n * 2 * real_bytes;
}

// Opt in to large dynamic shared memory on the current device.
cudaError_t line_filter_prepare() {
  cudaError_t e = cudaFuncSetAttribute(k_line_filter<float>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, kLineSmemMax);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_line_filter<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              kLineSmemMax);
}

template <typename R>
cudaError_t launch_line_filter(const AxisPlan &ap, const R *in, long long in_bstride, R *out,
                               long long out_bstride, const R *pre, const R *post,
                               long long w_bstride, int batch, cudaStream_t st) {
  const int n_pairs = (ap.n_real + 1) >> 1;
  dim3 grid((n_pairs + ap.tl - 1) / ap.tl, ap.n_outer, batch);
  const size_t smem = line_filter_smem_bytes(ap, sizeof(R));
  return launch_pdl(k_line_filter<R>, grid, dim3(256), smem, st, ap, in, in_bstride, out,
                    out_bstride, pre, post, w_bstride, static_cast<const PassDesc *>(nullptr));
}

cudaError_t launch_line_filter_desc(const AxisPlan &ap, const PassDesc *desc, int n,
                                    cudaStream_t st) {
  if (!desc || n < 1 || n > 65535 || ap.n_outer > 65535) return cudaErrorInvalidValue;
  const int n_pairs = (ap.n_real + 1) >> 1;
  dim3 grid((n_pairs + ap.tl - 1) / ap.tl, ap.n_outer, n);
  const size_t smem = line_filter_smem_bytes(ap, sizeof(float));
  return launch_pdl(k_line_filter<float>, grid, dim3(256), smem, st, ap,
                    static_cast<const float *>(nullptr), 0LL, static_cast<float *>(nullptr), 0LL,
                    static_cast<const float *>(nullptr), static_cast<const float *>(nullptr), 0LL,
                    desc);
}

template cudaError_t launch_line_filter<float>(const AxisPlan &, const float *, long long, float *,
                                               long long, const float *, const float *, long long,
                                               int, cudaStream_t);
template cudaError_t launch_line_filter<double>(const AxisPlan &, const double *, long long,
                                                double *, long long, const double *,
                                                const double *, long long, int, cudaStream_t);

}  // namespace scft
