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
__device__ __noinline__ C<T>* fft_lines(C<T>* a, C<T>* b, int nlines, int stride, const FftPlan& p,
                                        const C<T>* tw) {
  using V = C<T>;
  V* src = a;
  V* dst = b;
  const int n = p.n;
  for (int s = 0; s < p.nstages; ++s) {
    const int R = p.radix[s], Ns = p.ns[s], nb = n / R;
    const FastDiv dnb = p.dnb[s], dns = p.dns[s];
    const V* W = tw + p.tw_off[s];
    const int total = nlines * nb;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
      const int line = dnb.div(idx);
      const int j = idx - line * nb;
      const int k = j - dns.div(j) * Ns;
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
      } else if (R == 5) {
        V v0 = in[0], v1 = in[nb], v2 = in[2 * nb], v3 = in[3 * nb], v4 = in[4 * nb];
        if (k) {
          const V w1 = W[k], w2 = W[Ns + k], w3 = W[2 * Ns + k], w4 = W[3 * Ns + k];
          if (INV) {
            v1 = cmulc(v1, w1);
            v2 = cmulc(v2, w2);
            v3 = cmulc(v3, w3);
            v4 = cmulc(v4, w4);
          } else {
            v1 = cmul(v1, w1);
            v2 = cmul(v2, w2);
            v3 = cmul(v3, w3);
            v4 = cmul(v4, w4);
          }
        }
        // 5-point DFT from the symmetric and antisymmetric pairs:
        // cos(2 pi / 5), cos(4 pi / 5), sin(2 pi / 5), sin(4 pi / 5)
        const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;
        const T s1 = (T)0.95105651629515357212, s2 = (T)0.58778525229247312917;
        const V t1 = cadd(v1, v4), t2 = cadd(v2, v3), t3 = csub(v1, v4), t4 = csub(v2, v3);
        const V a1 = cmk<V>(v0.x + c1 * t1.x + c2 * t2.x, v0.y + c1 * t1.y + c2 * t2.y);
        const V a2 = cmk<V>(v0.x + c2 * t1.x + c1 * t2.x, v0.y + c2 * t1.y + c1 * t2.y);
        const V b1 = cmk<V>(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y);
        const V b2 = cmk<V>(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y);
        // forward: X1 = a1 - i b1, X4 = a1 + i b1, X2 = a2 - i b2, X3 = a2 + i b2
        const V mb1 = INV ? cmk<V>(-b1.y, b1.x) : cmk<V>(b1.y, -b1.x);  // -+ i b1
        const V mb2 = INV ? cmk<V>(-b2.y, b2.x) : cmk<V>(b2.y, -b2.x);
        out[0] = cadd(v0, cadd(t1, t2));
        out[Ns] = cadd(a1, mb1);
        out[2 * Ns] = cadd(a2, mb2);
        out[3 * Ns] = csub(a2, mb2);
        out[4 * Ns] = csub(a1, mb1);
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

// ------------------------------------------------------------ warp-level FFT
// 32nd roots of unity exp(-2 pi i k / 32), k = 0..15 (cos, -sin): cos(pi k / 16)
// and -sin(pi k / 16) to 20 digits.
__device__ __forceinline__ double w32_re(int k) {
  const double c[16] = {1.0,
                        0.98078528040323044913,
                        0.92387953251128675613,
                        0.83146961230254523708,
                        0.70710678118654752440,
                        0.55557023301960222474,
                        0.38268343236508977173,
                        0.19509032201612826785,
                        0.0,
                        -0.19509032201612826785,
                        -0.38268343236508977173,
                        -0.55557023301960222474,
                        -0.70710678118654752440,
                        -0.83146961230254523708,
                        -0.92387953251128675613,
                        -0.98078528040323044913};
  return c[k];
}
__device__ __forceinline__ double w32_im(int k) {
  const double s[16] = {0.0,
                        -0.19509032201612826785,
                        -0.38268343236508977173,
                        -0.55557023301960222474,
                        -0.70710678118654752440,
                        -0.83146961230254523708,
                        -0.92387953251128675613,
                        -0.98078528040323044913,
                        -1.0,
                        -0.98078528040323044913,
                        -0.92387953251128675613,
                        -0.83146961230254523708,
                        -0.70710678118654752440,
                        -0.55557023301960222474,
                        -0.38268343236508977173,
                        -0.19509032201612826785};
  return s[k];
}

// In-register DFT of N in {1, 2, 4, 8, 16, 32} values, natural order in and out,
// by radix-2 decimation in time.  INV uses the conjugate roots.
template <typename T, bool INV, int N>
struct RegDft {
  __device__ __forceinline__ static void run(C<T>* v) {
    using V = C<T>;
    V e[N / 2], o[N / 2];
#pragma unroll
    for (int i = 0; i < N / 2; ++i) {
      e[i] = v[2 * i];
      o[i] = v[2 * i + 1];
    }
    RegDft<T, INV, N / 2>::run(e);
    RegDft<T, INV, N / 2>::run(o);
#pragma unroll
    for (int k = 0; k < N / 2; ++k) {
      V t;
      if (k == 0) {
        t = o[k];
      } else if (4 * k == N) {  // multiply by -i (forward) or +i (inverse)
        t = INV ? cmk<V>(-o[k].y, o[k].x) : cmk<V>(o[k].y, -o[k].x);
      } else {
        const T wr = (T)w32_re(k * (32 / N));
        const T wi = INV ? (T)-w32_im(k * (32 / N)) : (T)w32_im(k * (32 / N));
        t = cmk<V>(o[k].x * wr - o[k].y * wi, o[k].x * wi + o[k].y * wr);
      }
      v[k] = cadd(e[k], t);
      v[k + N / 2] = csub(e[k], t);
    }
  }
};
template <typename T, bool INV>
struct RegDft<T, INV, 1> {
  __device__ __forceinline__ static void run(C<T>*) {}
};

// One line of length N = A * B owned by B lanes of one warp (lane b of the
// group), with the input already in registers: v[a] = x[b + B a].
//   x[b + B a] --(A-point DFT over a)--> Y[b][ka] --(* W_N^(b ka))-->
//   transpose in the line --(B-point DFT over b)--> X[ka + A kb].
// Lp is the line in shared memory, used for the transpose; it holds X in
// natural order on return.  All lanes of the warp must call it (inactive
// groups with active = false); `roots` holds exp(-2 pi i j / N), j < N.
// The transpose goes through rows of B + 1 elements when PAD (row ka at
// ka (B + 1): every address is the lane's base plus a compile-time offset,
// and the line then needs N + A - 1 elements of room), else through rows of
// B with the columns rotated by ka (N elements of room).
template <typename T, bool INV, int A, int B, bool PAD = false>
__device__ __forceinline__ void fft_line_regs(C<T> (&v)[A], C<T>* Lp, int b, bool active, const C<T>* roots) {
  using V = C<T>;
  constexpr int Q = A / B;
  RegDft<T, INV, A>::run(v);
#pragma unroll
  for (int ka = 1; ka < A; ++ka) {
    const V w = roots[b * ka];
    v[ka] = INV ? cmulc(v[ka], w) : cmul(v[ka], w);
  }
  __syncwarp();
  if (active) {
    if constexpr (PAD) {
      C<T>* row = Lp + b;
#pragma unroll
      for (int ka = 0; ka < A; ++ka) row[ka * (B + 1)] = v[ka];
    } else {
#pragma unroll
      for (int ka = 0; ka < A; ++ka) Lp[ka * B + ((b + ka) & (B - 1))] = v[ka];
    }
  }
  __syncwarp();
  // v is dead after the transpose: reuse it for the columns
  if (active) {
    if constexpr (PAD) {
      const C<T>* col = Lp + b * Q * (B + 1);
#pragma unroll
      for (int t = 0; t < Q; ++t)
#pragma unroll
        for (int bb = 0; bb < B; ++bb) v[t * B + bb] = col[t * (B + 1) + bb];
    } else {
#pragma unroll
      for (int t = 0; t < Q; ++t) {
        const int ka = b * Q + t;
#pragma unroll
        for (int bb = 0; bb < B; ++bb) v[t * B + bb] = Lp[ka * B + ((bb + ka) & (B - 1))];
      }
    }
  }
#pragma unroll
  for (int t = 0; t < Q; ++t) RegDft<T, INV, B>::run(v + t * B);
  __syncwarp();
  if (active) {
#pragma unroll
    for (int t = 0; t < Q; ++t)
#pragma unroll
      for (int kb = 0; kb < B; ++kb) Lp[(b * Q + t) + A * kb] = v[t * B + kb];
  }
  __syncwarp();
}

// Transforms `nlines` lines of length N = A * B in place (line l at
// buf + l * stride, stride >= N + A - 1 when PAD), 32 / B lines per warp at
// a time; only __syncwarp is needed inside.
template <typename T, bool INV, int A, int B, bool PAD = false>
__device__ __forceinline__ void fft_lines_warp_body(C<T>* buf, int nlines, int stride, const C<T>* roots) {
  using V = C<T>;
  constexpr int GPW = 32 / B;  // lines per warp
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int grp = lane / B, b = lane - grp * B;
  for (int line0 = warp * GPW; line0 < nlines; line0 += nwarps * GPW) {
    const int line = line0 + grp;
    const bool active = line < nlines;
    V* Lp = buf + (long long)(active ? line : 0) * stride;
    V v[A];
    if (active) {
#pragma unroll
      for (int a = 0; a < A; ++a) v[a] = Lp[b + B * a];
    }
    fft_line_regs<T, INV, A, B, PAD>(v, Lp, b, active, roots);
  }
}

// Out-of-line copy (kernels that hold much state around the transform call it
// so that the transform's registers are not added to theirs).
template <typename T, bool INV, int A, int B, bool PAD = false>
__device__ __noinline__ void fft_lines_warp(C<T>* buf, int nlines, int stride, const C<T>* roots) {
  fft_lines_warp_body<T, INV, A, B, PAD>(buf, nlines, stride, roots);
}

// ------------------------------------------------------ per-thread DFT
// A whole short line (N <= 16) in one thread's registers, by mixed-radix
// decimation in time with every index known at compile time: N = F M with F
// the smallest prime factor, X[k1 + M k2] = DFT_F over f of
// W_N^(f k1) Y_f[k1], Y_f = DFT_M(x[F m + f]).  Radix 2, 3, 4 and 5
// butterflies are written out; other primes are direct DFTs.  Roots:
// rt[j * RS] = exp(-2 pi i j / N) (a table of N * RS roots in shared memory).
template <int N>
struct SmallFactor {
  static constexpr int value = N % 4 == 0 ? 4 : N % 2 == 0 ? 2 : N % 3 == 0 ? 3 : N % 5 == 0 ? 5 : N % 7 == 0 ? 7 : N;
};

template <typename T, bool INV, int N, int RS>
struct ThreadDft {
  __device__ __forceinline__ static void run(C<T>* v, const C<T>* rt) {
    using V = C<T>;
    constexpr int F = SmallFactor<N>::value, M = N / F;
    if constexpr (M == 1) {
      butterfly(v, rt);
    } else {
      V sub[F][M];
#pragma unroll
      for (int f = 0; f < F; ++f)
#pragma unroll
        for (int m = 0; m < M; ++m) sub[f][m] = v[F * m + f];
#pragma unroll
      for (int f = 0; f < F; ++f) ThreadDft<T, INV, M, RS * F>::run(sub[f], rt);
#pragma unroll
      for (int k1 = 0; k1 < M; ++k1) {
        V z[F];
#pragma unroll
        for (int f = 0; f < F; ++f) {
          const int e = (f * k1) % N;
          if (e == 0) {
            z[f] = sub[f][k1];
          } else {
            const V w = rt[e * RS];
            z[f] = INV ? cmulc(sub[f][k1], w) : cmul(sub[f][k1], w);
          }
        }
        ThreadDft<T, INV, F, RS * M>::run(z, rt);
#pragma unroll
        for (int k2 = 0; k2 < F; ++k2) v[k1 + M * k2] = z[k2];
      }
    }
  }
  // N prime or 4: the butterfly on v[0..N)
  __device__ __forceinline__ static void butterfly(C<T>* v, const C<T>* rt) {
    using V = C<T>;
    if constexpr (N == 2) {
      const V a = v[0], b = v[1];
      v[0] = cadd(a, b);
      v[1] = csub(a, b);
    } else if constexpr (N == 4) {
      const V a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]), a2 = cadd(v[1], v[3]), a3 = csub(v[1], v[3]);
      const V r3 = INV ? cmk<V>(-a3.y, a3.x) : cmk<V>(a3.y, -a3.x);
      v[0] = cadd(a0, a2);
      v[1] = cadd(a1, r3);
      v[2] = csub(a0, a2);
      v[3] = csub(a1, r3);
    } else if constexpr (N == 3) {
      const T s3 = (T)0.86602540378443864676;  // sin(2 pi / 3)
      const V v0 = v[0], t1 = cadd(v[1], v[2]), t3 = csub(v[1], v[2]);
      const V t2 = cmk<V>(v0.x - (T)0.5 * t1.x, v0.y - (T)0.5 * t1.y);
      const V r = INV ? cmk<V>(-s3 * t3.y, s3 * t3.x) : cmk<V>(s3 * t3.y, -s3 * t3.x);
      v[0] = cadd(v0, t1);
      v[1] = cadd(t2, r);
      v[2] = csub(t2, r);
    } else if constexpr (N == 5) {
      const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;
      const T s1 = (T)0.95105651629515357212, s2 = (T)0.58778525229247312917;
      const V v0 = v[0];
      const V t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]), t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
      const V a1 = cmk<V>(v0.x + c1 * t1.x + c2 * t2.x, v0.y + c1 * t1.y + c2 * t2.y);
      const V a2 = cmk<V>(v0.x + c2 * t1.x + c1 * t2.x, v0.y + c2 * t1.y + c1 * t2.y);
      const V b1 = cmk<V>(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y);
      const V b2 = cmk<V>(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y);
      const V mb1 = INV ? cmk<V>(-b1.y, b1.x) : cmk<V>(b1.y, -b1.x);
      const V mb2 = INV ? cmk<V>(-b2.y, b2.x) : cmk<V>(b2.y, -b2.x);
      v[0] = cadd(v0, cadd(t1, t2));
      v[1] = cadd(a1, mb1);
      v[2] = cadd(a2, mb2);
      v[3] = csub(a2, mb2);
      v[4] = csub(a1, mb1);
    } else {  // other primes: direct DFT
      V x[N];
#pragma unroll
      for (int j = 0; j < N; ++j) x[j] = v[j];
#pragma unroll
      for (int k = 0; k < N; ++k) {
        V acc = x[0];
#pragma unroll
        for (int j = 1; j < N; ++j) {
          const int e = (j * k) % N;
          if (e == 0) {
            acc = cadd(acc, x[j]);
          } else {
            const V w = rt[e * RS];
            acc = cadd(acc, INV ? cmulc(x[j], w) : cmul(x[j], w));
          }
        }
        v[k] = acc;
      }
    }
  }
};
template <typename T, bool INV, int RS>
struct ThreadDft<T, INV, 1, RS> {
  __device__ __forceinline__ static void run(C<T>*, const C<T>*) {}
};

// Transform dispatcher: the warp-level path for the lengths the plan marks,
// the Stockham stages otherwise.  Returns the buffer holding the result; all
// threads of the block must call it after the input is complete
// (__syncthreads()), and the result is complete for all threads on return.
template <typename T, bool INV, int A, int B, bool INL, bool PAD = false>
__device__ __forceinline__ void fft_warp_call(C<T>* buf, int nlines, int stride, const C<T>* roots) {
  if constexpr (INL)
    fft_lines_warp_body<T, INV, A, B, PAD>(buf, nlines, stride, roots);
  else
    fft_lines_warp<T, INV, A, B, PAD>(buf, nlines, stride, roots);
}

// INL: expand the warp-level transforms into the calling kernel.
// WIDE: also the 32-value shapes (lengths 512 and 1024).  They need about
// twice the registers, and a kernel's register allocation covers everything
// it calls, so only kernels instantiated with WIDE = true contain them; a
// plan with warp_a == 32 must only reach those (the host checks).
// PAD: the warp-level transforms use padded transpose rows (stride >=
// n + warp_a - 1).
template <typename T, bool INV, bool INL = false, bool WIDE = false, bool PAD = false>
__device__ C<T>* fft_run(C<T>* a, C<T>* b, int nlines, int stride, const FftPlan& p, const C<T>* tw) {
  if constexpr (WIDE) {
    if (p.warp_a == 32) {
      if (p.warp_b == 32)
        fft_warp_call<T, INV, 32, 32, INL, PAD>(a, nlines, stride, tw + p.full_off);
      else
        fft_warp_call<T, INV, 32, 16, INL, PAD>(a, nlines, stride, tw + p.full_off);
      __syncthreads();
      return a;
    }
  }
  if (p.warp_a == 16 && p.warp_b == 16) {
    fft_warp_call<T, INV, 16, 16, INL, PAD>(a, nlines, stride, tw + p.full_off);
  } else if (p.warp_a == 16 && p.warp_b == 8) {
    fft_warp_call<T, INV, 16, 8, INL, PAD>(a, nlines, stride, tw + p.full_off);
  } else if (p.warp_a == 8 && p.warp_b == 8) {
    fft_warp_call<T, INV, 8, 8, INL, PAD>(a, nlines, stride, tw + p.full_off);
  } else if (p.warp_a == 16 && p.warp_b == 2) {
    fft_warp_call<T, INV, 16, 2, INL, PAD>(a, nlines, stride, tw + p.full_off);
  } else if (p.warp_a == 8 && p.warp_b == 4) {
    fft_warp_call<T, INV, 8, 4, INL, PAD>(a, nlines, stride, tw + p.full_off);
  } else {
    return fft_lines<T, INV>(a, b, nlines, stride, p, tw);
  }
  __syncthreads();
  return a;
}

}  // namespace mmc
