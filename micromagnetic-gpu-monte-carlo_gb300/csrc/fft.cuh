// fft.cuh -- batched mixed-radix Stockham FFT on lines held in shared memory.
//
// The reference ran cuFFT (src/main.cu:593-675, 868-877).  Here every
// transform is a hand-written autosort (Stockham) FFT over a batch of lines in
// shared memory, so that a pass kernel can load a tile, transform it, apply
// the tensor product and transform back without leaving the SM.  Stage s of a
// length-n transform with radix R and span Ns reads element j + t*(n/R) of the
// source, multiplies by exp(-+2 pi i t k/(Ns R)), k = j mod Ns, does an R-point
// DFT and writes element (j-k)*R + k + q*Ns of the destination.
#pragma once
#include "mmc_internal.h"

namespace mmc {

template <typename T>
struct Cplx;
template <>
struct Cplx<float> {
  using type = float2;
};
template <>
struct Cplx<double> {
  using type = double2;
};
template <typename T>
using C = typename Cplx<T>::type;

template <typename V>
__device__ __forceinline__ V cmk(decltype(V::x) a, decltype(V::x) b) {
  V r;
  r.x = a;
  r.y = b;
  return r;
}
template <typename V>
__device__ __forceinline__ V cadd(V a, V b) {
  return cmk<V>(a.x + b.x, a.y + b.y);
}
template <typename V>
__device__ __forceinline__ V csub(V a, V b) {
  return cmk<V>(a.x - b.x, a.y - b.y);
}
template <typename V>
__device__ __forceinline__ V cmul(V a, V b) {
  return cmk<V>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename V>
__device__ __forceinline__ V cmulc(V a, V b) {
  return cmk<V>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

template <typename T>
__device__ __forceinline__ const C<T>* plan_tw(const FftPlan& p);
template <>
__device__ __forceinline__ const float2* plan_tw<float>(const FftPlan& p) {
  return p.tw32;
}
template <>
__device__ __forceinline__ const double2* plan_tw<double>(const FftPlan& p) {
  return p.tw64;
}

// Copies the plan's twiddle table into shared memory (call before the FFT,
// followed by __syncthreads()).
template <typename T>
__device__ __forceinline__ void load_twiddles(const FftPlan& p, C<T>* dst) {
  const C<T>* src = plan_tw<T>(p);
  for (int i = threadIdx.x; i < p.tw_total; i += blockDim.x) dst[i] = src[i];
}

// Transforms `nlines` lines of length p.n; line l starts at buf + l*stride.
// `a` holds the input, `b` is scratch of the same shape.  Returns the buffer
// holding the result (a or b).  All threads of the block must call it.
template <typename T, bool INV>
__device__ C<T>* fft_lines(C<T>* a, C<T>* b, int nlines, int stride, const FftPlan& p, const C<T>* tw) {
  using V = C<T>;
  V* src = a;
  V* dst = b;
  const int n = p.n;
  for (int s = 0; s < p.nstages; ++s) {
    const int R = p.radix[s], Ns = p.ns[s], nb = n / R;
    const V* W = tw + p.tw_off[s];
    const int total = nlines * nb;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
      const int line = idx / nb;
      const int j = idx - line * nb;
      const int k = j % Ns;
      const V* in = src + (long long)line * stride + j;
      V* out = dst + (long long)line * stride + (j - k) * R + k;
      if (R == 4) {
        V v0 = in[0], v1 = in[nb], v2 = in[2 * nb], v3 = in[3 * nb];
        if (k) {
          V w1 = W[k], w2 = W[Ns + k], w3 = W[2 * Ns + k];
          if (INV) {
            v1 = cmulc(v1, w1);
            v2 = cmulc(v2, w2);
            v3 = cmulc(v3, w3);
          } else {
            v1 = cmul(v1, w1);
            v2 = cmul(v2, w2);
            v3 = cmul(v3, w3);
          }
        }
        V a0 = cadd(v0, v2), a1 = csub(v0, v2), a2 = cadd(v1, v3), a3 = csub(v1, v3);
        V r3 = INV ? cmk<V>(-a3.y, a3.x) : cmk<V>(a3.y, -a3.x);
        out[0] = cadd(a0, a2);
        out[Ns] = cadd(a1, r3);
        out[2 * Ns] = csub(a0, a2);
        out[3 * Ns] = csub(a1, r3);
      } else if (R == 2) {
        V v0 = in[0], v1 = in[nb];
        if (k) v1 = INV ? cmulc(v1, W[k]) : cmul(v1, W[k]);
        out[0] = cadd(v0, v1);
        out[Ns] = csub(v0, v1);
      } else if (R == 3) {
        V v0 = in[0], v1 = in[nb], v2 = in[2 * nb];
        if (k) {
          V w1 = W[k], w2 = W[Ns + k];
          if (INV) {
            v1 = cmulc(v1, w1);
            v2 = cmulc(v2, w2);
          } else {
            v1 = cmul(v1, w1);
            v2 = cmul(v2, w2);
          }
        }
        const T s3 = (T)0.86602540378443864676;  // sin(2 pi / 3)
        V t1 = cadd(v1, v2);
        V t2 = cmk<V>(v0.x - (T)0.5 * t1.x, v0.y - (T)0.5 * t1.y);
        V t3 = csub(v1, v2);
        V r = INV ? cmk<V>(-s3 * t3.y, s3 * t3.x) : cmk<V>(s3 * t3.y, -s3 * t3.x);
        out[0] = cadd(v0, t1);
        out[Ns] = cadd(t2, r);
        out[2 * Ns] = csub(t2, r);
      } else {
        // generic odd radix: direct R-point DFT with the stage's roots of unity
        const V* RT = tw + p.root_off[s];
        V v[FFT_MAX_RADIX];
        for (int t = 0; t < R; ++t) {
          V x = in[t * nb];
          if (t && k) x = INV ? cmulc(x, W[(t - 1) * Ns + k]) : cmul(x, W[(t - 1) * Ns + k]);
          v[t] = x;
        }
        for (int q = 0; q < R; ++q) {
          V acc = v[0];
          int e = 0;
          for (int t = 1; t < R; ++t) {
            e += q;
            if (e >= R) e -= R;
            acc = INV ? cadd(acc, cmulc(v[t], RT[e])) : cadd(acc, cmul(v[t], RT[e]));
          }
          out[q * Ns] = acc;
        }
      }
    }
    __syncthreads();
    V* t = src;
    src = dst;
    dst = t;
  }
  return src;
}

}  // namespace mmc
