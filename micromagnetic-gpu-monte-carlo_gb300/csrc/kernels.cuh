// kernels.cuh -- demag convolution passes, Metropolis sweep, energy and field
// kernels, templated on the working precision T (float or double).
//
// Included by kernels_f32.cu (built with multiply-add contraction) and
// kernels_f64.cu (built with -fmad=false so that FP64 results match the CPU
// oracle bit for bit where the operation order is the same).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>

#include "fft.cuh"
#include "mmc_internal.h"
#include "mmc_math.h"

namespace mmc {

// =========================================================== launch helpers
// Programmatic dependent launch: a kernel launched by launch_pdl may be
// scheduled before the previous kernel of its stream (or graph branch) has
// retired, and calls pdl_wait() before it reads anything a previous kernel
// writes or writes anything one reads; before the wait it touches only
// constant tables (transform roots and twiddles).  The previous kernels
// trigger implicitly when their CTAs exit: an explicit early trigger let the
// next grid's waiting CTAs take SM slots during the tail and cost 4 us per
// batched sweep.  The wait returns at once for a kernel launched without the
// attribute.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, args...);
}

// =========================================================== demag passes
//
// The reference computes H^ = K^ . M^ / N with three cuFFT R2C transforms and
// calHexchangeKernel (src/main.cu:868-884, src/demag_cu.cu:68-116) and never
// runs the inverse.  Here the convolution is complete and split into
//   x_forward : real rows -> half spectrum along x (two real rows per complex FFT)
//   col_pass  : complex FFT along y or z over tiles of kx columns, optionally
//               fused with the 3x3 tensor product and the inverse FFT
//   x_inverse : half spectrum -> real rows, cropped to the lattice
// Rows that are pure zero padding are never loaded (pruned transform).

// Real rows in[c][row][x] (x < xdata, zero up to p.n) -> S[c][z][y][kx], kx < hx.
// NC: components (3 for m, 6 for the tensor), fixed at compile time so the
// per-element work covers only the components that exist.
template <typename T, bool INL, int NC>
__global__ void k_x_forward(FftPlan p, int xdata, FastDiv dyd, int nrows, const T* __restrict__ in,
                            long long in_cstride, C<T>* __restrict__ S, long long nspec, int nyp, FastDiv dhx,
                            int pitch, int rows_per_cta, long long in_rstride, long long s_rstride) {
  constexpr int ncomp = NC;
  const int hx = (int)dhx.d, ydata = (int)dyd.d;
  using V = C<T>;
  in += blockIdx.z * in_rstride;  // replica of a batch
  S += blockIdx.z * s_rstride;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* tw = reinterpret_cast<V*>(smem_raw);
  const int L = p.n;
  constexpr int npairs = (ncomp + 1) / 2;
  const int row0 = blockIdx.x * rows_per_cta;
  const int nr = min(rows_per_cta, nrows - row0);
  V* bufA = tw + ((p.tw_total + 1) & ~1);
  V* bufB = bufA + (long long)rows_per_cta * npairs * L;
  load_twiddles<T>(p, tw);
  // loads are issued four elements per thread at a time, before any store, so
  // their latencies overlap
  const int total = nr * L;
  for (int base = threadIdx.x; base < total; base += 4 * blockDim.x) {
    T v[4][2 * npairs];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int idx = base + u * blockDim.x;
      const int rr = p.dn.div(idx), x = idx - rr * L;
      const bool ok = idx < total && x < xdata;
      const long long rbase = (long long)(row0 + rr) * xdata + x;
#pragma unroll
      for (int c = 0; c < 2 * npairs; ++c) v[u][c] = (ok && c < ncomp) ? in[c * in_cstride + rbase] : (T)0;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int idx = base + u * blockDim.x;
      if (idx < total) {
        const int rr = p.dn.div(idx), x = idx - rr * L;
#pragma unroll
        for (int pr = 0; pr < npairs; ++pr)
          bufA[(long long)(rr * npairs + pr) * L + x] = cmk<V>(v[u][2 * pr], v[u][2 * pr + 1]);
      }
    }
  }
  __syncthreads();
  V* res = fft_run<T, false, INL, NC == 6>(bufA, bufB, nr * npairs, L, p, tw);
  for (int idx = threadIdx.x; idx < nr * npairs * hx; idx += blockDim.x) {
    const int rest = dhx.div(idx);
    const int k = idx - rest * hx;
    const int rr = rest / npairs, pr = rest - rr * npairs;  // npairs is a compile-time 2 or 3
    const V* line = res + (long long)(rr * npairs + pr) * L;
    const V A = line[k];
    const V B = line[k == 0 ? 0 : L - k];
    const int row = row0 + rr;
    const int z = dyd.div(row), y = row - z * ydata;
    const long long off = ((long long)z * nyp + y) * pitch + k;
    const int ca = 2 * pr, cb = 2 * pr + 1;
    S[ca * nspec + off] = cmk<V>((T)0.5 * (A.x + B.x), (T)0.5 * (A.y - B.y));
    if (cb < ncomp) S[cb * nspec + off] = cmk<V>((T)0.5 * (A.y + B.y), (T)-0.5 * (A.x - B.x));
  }
}

// Half spectra S[0..2][z][y][kx] -> real rows out[c][row][x], x < xout.
template <typename T, bool INL>
__global__ void k_x_inverse(FftPlan p, const C<T>* __restrict__ S, long long nspec, int nyp, int hx, int pitch,
                            FastDiv dxo, FastDiv dyo, int nrows, T* __restrict__ out, long long out_cstride,
                            int rows_per_cta, long long s_rstride, long long out_rstride) {
  const int xout = (int)dxo.d, yout = (int)dyo.d;
  using V = C<T>;
  S += blockIdx.z * s_rstride;
  out += blockIdx.z * out_rstride;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* tw = reinterpret_cast<V*>(smem_raw);
  const int L = p.n;
  const int row0 = blockIdx.x * rows_per_cta;
  const int nr = min(rows_per_cta, nrows - row0);
  V* bufA = tw + ((p.tw_total + 1) & ~1);
  V* bufB = bufA + (long long)rows_per_cta * 2 * L;
  load_twiddles<T>(p, tw);
  const int total = nr * L;
  for (int base0 = threadIdx.x; base0 < total; base0 += 4 * blockDim.x) {
    V v[4][3];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int idx = base0 + u * blockDim.x;
      const int rr = p.dn.div(idx), k = idx - rr * L;
      const int row = row0 + rr;
      const int z = dyo.div(row), y = row - z * yout;
      const long long base = ((long long)z * nyp + y) * pitch;
      const long long kk = k < hx ? k : L - k;
#pragma unroll
      for (int c = 0; c < 3; ++c) v[u][c] = idx < total ? S[c * nspec + base + kk] : cmk<V>(0, 0);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int idx = base0 + u * blockDim.x;
      if (idx < total) {
        const int rr = p.dn.div(idx), k = idx - rr * L;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          if (k >= hx) v[u][c].y = -v[u][c].y;
          if (k == 0 || 2 * k == L) v[u][c].y = 0;  // bins that are real for a real output
        }
        bufA[(long long)(rr * 2) * L + k] = cmk<V>(v[u][0].x - v[u][1].y, v[u][0].y + v[u][1].x);
        bufA[(long long)(rr * 2 + 1) * L + k] = v[u][2];
      }
    }
  }
  __syncthreads();
  V* res = fft_run<T, true, INL>(bufA, bufB, nr * 2, L, p, tw);
  for (int idx = threadIdx.x; idx < nr * xout; idx += blockDim.x) {
    const int rr = dxo.div(idx), x = idx - rr * xout;
    const long long o = (long long)(row0 + rr) * xout + x;
    const V a = res[(long long)(rr * 2) * L + x];
    const V b = res[(long long)(rr * 2 + 1) * L + x];
    out[o] = a.x;
    out[out_cstride + o] = a.y;
    out[2 * out_cstride + o] = b.x;
  }
}

// ----------------------------------------------------- warp-shaped x passes
// The same two transforms for lengths with a warp-level plan (L = A * B):
// each line (a pair of components of one row) goes straight from global
// memory into the registers of its B lanes in the order the transform takes
// it (element b + B a in lane b of the group), so the input is never staged
// in shared memory, and the loops over rows and columns need no division.
// Same arithmetic as k_x_forward / k_x_inverse, so the results are the same
// bit for bit.  Shared memory: the L roots and one L-element line per
// (row, pair).
template <typename T>
__device__ __forceinline__ void load_roots(const FftPlan& p, C<T>* dst) {
  const C<T>* src = plan_tw<T>(p) + p.full_off;
  for (int i = threadIdx.x; i < p.n; i += blockDim.x) dst[i] = src[i];
}

// (Register budget: 64 per thread in FP32 with 16 values per lane, so that
// eight 128-thread CTAs fit on an SM; twice that in FP64 or with 32 values.)
template <typename T, int A>
constexpr int x_w_min_blocks() {
  return (sizeof(T) == 4 ? 4 : 2) / (A >= 32 ? 2 : 1);
}
template <typename T, int A, int B>
__global__ void __launch_bounds__(256, x_w_min_blocks<T, A>()) k_x_forward_w(FftPlan p, int xdata, FastDiv dyd, int nrows, const T* __restrict__ in,
                              long long in_cstride, C<T>* __restrict__ S, long long nspec, int nyp, int hx,
                              int pitch, int rows_per_cta, long long in_rstride, long long s_rstride) {
  constexpr int L = A * B, GPW = 32 / B;
  using V = C<T>;
  const int ydata = (int)dyd.d;
  in += blockIdx.z * in_rstride;
  S += blockIdx.z * s_rstride;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int LS = L + A;  // line stride: room for the padded transpose
  V* roots = reinterpret_cast<V*>(smem_raw);
  V* buf = roots + L;  // line pr * nr + rr: row rr, pair pr (mx + i my, mz + 0 i)
  load_roots<T>(p, roots);
  pdl_wait();
  __syncthreads();
  const int row0 = blockIdx.x * rows_per_cta;
  const int nr = min(rows_per_cta, nrows - row0);
  const int nlines = 2 * nr;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int grp = lane / B, b = lane - grp * B;
  // pair-major line order: the groups of a warp mostly load the same pair
  for (int line0 = warp * GPW; line0 < nlines; line0 += nwarps * GPW) {
    const int line = line0 + grp;
    const bool active = line < nlines;
    const int pr = line >= nr ? 1 : 0, rr = line - pr * nr;
    V v[A];
    if (active) {
      const T* re = in + (long long)(2 * pr) * in_cstride + (long long)(row0 + rr) * xdata;
#pragma unroll
      for (int a = 0; a < A; ++a) {
        const int x = b + B * a;
        const bool ok = x < xdata;
        v[a] = cmk<V>(ok ? re[x] : (T)0, (ok && pr == 0) ? re[in_cstride + x] : (T)0);
      }
    }
    fft_line_regs<T, false, A, B, true>(v, buf + (active ? line : 0) * LS, b, active, roots);
  }
  __syncthreads();
  // split each pair into the half spectra of its two real rows
  for (int line = warp; line < nlines; line += nwarps) {
    const int pr = line >= nr ? 1 : 0, rr = line - pr * nr;
    const V* ln = buf + line * LS;
    const int row = row0 + rr;
    const int z = dyd.div(row), y = row - z * ydata;
    V* so = S + (long long)(2 * pr) * nspec + ((long long)z * nyp + y) * pitch;
    for (int k = lane; k < hx; k += 32) {
      const V Av = ln[k];
      const V Bv = ln[k == 0 ? 0 : L - k];
      so[k] = cmk<V>((T)0.5 * (Av.x + Bv.x), (T)0.5 * (Av.y - Bv.y));
      if (pr == 0) so[nspec + k] = cmk<V>((T)0.5 * (Av.y + Bv.y), (T)-0.5 * (Av.x - Bv.x));
    }
  }
}

template <typename T, int A, int B>
__global__ void __launch_bounds__(256, x_w_min_blocks<T, A>()) k_x_inverse_w(FftPlan p, const C<T>* __restrict__ S, long long nspec, int nyp, int hx, int pitch,
                              FastDiv dxo, FastDiv dyo, int nrows, T* __restrict__ out, long long out_cstride,
                              int rows_per_cta, long long s_rstride, long long out_rstride) {
  constexpr int L = A * B, GPW = 32 / B;
  using V = C<T>;
  const int xout = (int)dxo.d, yout = (int)dyo.d;
  S += blockIdx.z * s_rstride;
  out += blockIdx.z * out_rstride;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int LS = L + A;  // line stride: room for the padded transpose
  V* roots = reinterpret_cast<V*>(smem_raw);
  V* buf = roots + L;  // line rr: hx + i hy of row rr; line nr + rr: hz
  load_roots<T>(p, roots);
  pdl_wait();
  __syncthreads();
  const int row0 = blockIdx.x * rows_per_cta;
  const int nr = min(rows_per_cta, nrows - row0);
  const int nlines = 2 * nr;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int grp = lane / B, b = lane - grp * B;
  for (int line0 = warp * GPW; line0 < nlines; line0 += nwarps * GPW) {
    const int line = line0 + grp;
    const bool active = line < nlines;
    const int pr = line >= nr ? 1 : 0, rr = line - pr * nr;
    V v[A];
    if (active) {
      const int row = row0 + rr;
      const int z = dyo.div(row), y = row - z * yout;
      const V* si = S + (long long)(2 * pr) * nspec + ((long long)z * nyp + y) * pitch;
#pragma unroll
      for (int a = 0; a < A; ++a) {
        const int k = b + B * a;
        const int kk = k < hx ? k : L - k;
        V u0 = si[kk];
        if (k >= hx) u0.y = -u0.y;
        if (k == 0 || 2 * k == L) u0.y = 0;  // bins that are real for a real output
        if (pr == 0) {
          V u1 = si[nspec + kk];
          if (k >= hx) u1.y = -u1.y;
          if (k == 0 || 2 * k == L) u1.y = 0;
          v[a] = cmk<V>(u0.x - u1.y, u0.y + u1.x);
        } else {
          v[a] = u0;
        }
      }
    }
    fft_line_regs<T, true, A, B, true>(v, buf + (active ? line : 0) * LS, b, active, roots);
  }
  __syncthreads();
  for (int rr = warp; rr < nr; rr += nwarps) {
    const V* l0 = buf + rr * LS;
    const V* l1 = buf + (nr + rr) * LS;
    T* o = out + (long long)(row0 + rr) * xout;
    for (int x = lane; x < xout; x += 32) {
      const V a = l0[x];
      o[x] = a.x;
      o[out_cstride + x] = a.y;
      o[2 * out_cstride + x] = l1[x].x;
    }
  }
}

// PASS_SYM (with PASS_MUL): multiply by the real part of K^ only, i.e. by the
// spectrum of (K(r) + K(-r)) / 2 -- the symmetrised tensor of the energy's
// adjoint.
enum : int { PASS_FWD = 1, PASS_MUL = 2, PASS_INV = 4, PASS_SYM = 8 };

// Complex FFT along a strided axis (y or z) of tiles of `tx` consecutive kx
// columns.  Element (c, pos, col) lives at S[c*nspec + plane*plane_stride +
// pos*pos_stride + kx0 + col].  Loads pos < load_lim (zero above), stores
// pos < store_lim.  With PASS_MUL the tile is multiplied by the symmetric
// tensor spectrum (K^ . M^ / N, calHexchangeKernel) between the transforms.
template <typename T, bool INL, bool WIDE>
__device__ __forceinline__ void col_pass_body(const FftPlan& p, int ncomp, C<T>* __restrict__ S, long long nspec,
                                              const C<T>* __restrict__ khat, int hx, long long plane_stride,
                                              long long pos_stride, int load_lim, int store_lim, int flags, T inv_n,
                                              int tx, long long s_rstride, int lean) {
  using V = C<T>;
  S += blockIdx.z * s_rstride;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* tw = reinterpret_cast<V*>(smem_raw);
  const int L = p.n;
  const int stride = col_line_stride(p, sizeof(V));
  const int kx0 = blockIdx.x * tx;
  const int ntx = min(tx, hx - kx0);
  const long long pbase = (long long)blockIdx.y * plane_stride + kx0;
  const int nlines = ncomp * ntx;
  // lean 1 (warp-level transforms only): one buffer, transformed in place,
  // and the tensor read from global memory in the product -- a third of the
  // shared memory, so more CTAs fit on an SM.  lean 2: two buffers, the tensor
  // read from global memory (lines too long for the staged tensor tile).
  V* bufA = tw + ((p.tw_total + 1) & ~1);
  V* bufB = lean == 1 ? bufA : bufA + (long long)ncomp * tx * stride;
  V* ktile = bufB + (long long)ncomp * tx * stride;  // [comp][pos][t] when PASS_MUL and not lean
  load_twiddles<T>(p, tw);
  // the tensor tile goes to shared memory asynchronously while the forward
  // transform runs (16-byte copies when the tile rows are 16-byte aligned)
  const bool kasync = !lean && (flags & PASS_MUL) && (((long long)ntx * sizeof(V)) % 16 == 0) && ((kx0 * sizeof(V)) % 16 == 0) &&
                      ((plane_stride * sizeof(V)) % 16 == 0) && ((pos_stride * sizeof(V)) % 16 == 0);
  const FastDiv dt((uint32_t)ntx);  // index arithmetic without run-time division
  if ((flags & PASS_MUL) && !lean) {
    const int per = (int)(ntx * sizeof(V) / 16);
    if (kasync) {
      const FastDiv dper((uint32_t)per);
      for (int idx = threadIdx.x; idx < 6 * L * per; idx += blockDim.x) {
        const int rest = dper.div(idx), q = idx - rest * per;
        const int c = p.dn.div(rest), pos = rest - c * L;
        const int e = 16 / (int)sizeof(V);
        const unsigned sd = (unsigned)__cvta_generic_to_shared(ktile + ((long long)c * L + pos) * ntx + q * e);
        const V* src = khat + c * nspec + pbase + pos * pos_stride + q * e;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sd), "l"(src) : "memory");
      }
    } else {
      for (int idx = threadIdx.x; idx < 6 * L * ntx; idx += blockDim.x) {
        const int rest = dt.div(idx), t = idx - rest * ntx;
        const int c = p.dn.div(rest), pos = rest - c * L;
        ktile[((long long)c * L + pos) * ntx + t] = khat[c * nspec + pbase + pos * pos_stride + t];
      }
    }
  }
  pdl_wait();  // the spectrum is the previous pass's output
  // thread -> (column t, first position pos0); positions advance by pstep, so
  // the loops below need no division (tx is a power of two)
  const int lg = __ffs(tx) - 1;
  const int t = threadIdx.x & (tx - 1), pos0 = threadIdx.x >> lg, pstep = blockDim.x >> lg;
  const bool tok = t < ntx;
  constexpr int LB = 8;  // loads in flight per thread
  for (int c = 0; c < ncomp; ++c) {
    const V* src = S + c * nspec + pbase + t;
    V* dst = bufA + (long long)(c * ntx + t) * stride;
    for (int pos = pos0; pos < L; pos += LB * pstep) {
      V v[LB];
#pragma unroll
      for (int u = 0; u < LB; ++u) {
        const int q = pos + u * pstep;
        v[u] = (tok && q < load_lim) ? src[(long long)q * pos_stride] : cmk<V>(0, 0);
      }
#pragma unroll
      for (int u = 0; u < LB; ++u) {
        const int q = pos + u * pstep;
        if (tok && q < L) dst[q] = v[u];
      }
    }
  }
  __syncthreads();
  V* cur = bufA;
  V* oth = bufB;
  if (flags & PASS_FWD) {
    V* r = fft_run<T, false, INL, WIDE, true>(cur, oth, nlines, stride, p, tw);
    if (r != cur) {
      oth = cur;
      cur = r;
    }
  }
  if (flags & PASS_MUL) {
    if (kasync) asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
    for (int pos = pos0; tok && pos < L; pos += pstep) {
      const V* kk = lean ? khat + pbase + pos * pos_stride + t : ktile + (long long)pos * ntx + t;
      const long long ks = lean ? nspec : (long long)L * ntx;
      V kxx = kk[0], kxy = kk[ks], kxz = kk[2 * ks];
      V kyy = kk[3 * ks], kyz = kk[4 * ks], kzz = kk[5 * ks];
      if (flags & PASS_SYM) kxx.y = kxy.y = kxz.y = kyy.y = kyz.y = kzz.y = (T)0;
      V* px = cur + (long long)(0 * ntx + t) * stride + pos;
      V* py = cur + (long long)(1 * ntx + t) * stride + pos;
      V* pz = cur + (long long)(2 * ntx + t) * stride + pos;
      const V mx = *px, my = *py, mz = *pz;
      // src/demag_cu.cu:98-111: real and imaginary parts of sum_b K_ab M_b, divided by N
      T hxr = (mx.x * kxx.x - mx.y * kxx.y) + (my.x * kxy.x - my.y * kxy.y) + (mz.x * kxz.x - mz.y * kxz.y);
      T hxi = (mx.x * kxx.y + mx.y * kxx.x) + (my.x * kxy.y + my.y * kxy.x) + (mz.x * kxz.y + mz.y * kxz.x);
      T hyr = (mx.x * kxy.x - mx.y * kxy.y) + (my.x * kyy.x - my.y * kyy.y) + (mz.x * kyz.x - mz.y * kyz.y);
      T hyi = (mx.x * kxy.y + mx.y * kxy.x) + (my.x * kyy.y + my.y * kyy.x) + (mz.x * kyz.y + mz.y * kyz.x);
      T hzr = (mx.x * kxz.x - mx.y * kxz.y) + (my.x * kyz.x - my.y * kyz.y) + (mz.x * kzz.x - mz.y * kzz.y);
      T hzi = (mx.x * kxz.y + mx.y * kxz.x) + (my.x * kyz.y + my.y * kyz.x) + (mz.x * kzz.y + mz.y * kzz.x);
      *px = cmk<V>(hxr * inv_n, hxi * inv_n);
      *py = cmk<V>(hyr * inv_n, hyi * inv_n);
      *pz = cmk<V>(hzr * inv_n, hzi * inv_n);
    }
    __syncthreads();
  }
  if (flags & PASS_INV) {
    V* r = fft_run<T, true, INL, WIDE, true>(cur, oth, nlines, stride, p, tw);
    if (r != cur) {
      oth = cur;
      cur = r;
    }
  }
  if (tok) {
    for (int c = 0; c < ncomp; ++c) {
      V* dst = S + c * nspec + pbase + t;
      const V* src = cur + (long long)(c * ntx + t) * stride;
      for (int pos = pos0; pos < store_lim; pos += pstep) dst[(long long)pos * pos_stride] = src[pos];
    }
  }
}

template <typename T, bool INL>
__global__ void k_col_pass(FftPlan p, int ncomp, C<T>* __restrict__ S, long long nspec,
                           const C<T>* __restrict__ khat, int hx, long long plane_stride, long long pos_stride,
                           int load_lim, int store_lim, int flags, T inv_n, int tx, long long s_rstride, int lean) {
  col_pass_body<T, INL, false>(p, ncomp, S, nspec, khat, hx, plane_stride, pos_stride, load_lim, store_lim, flags,
                               inv_n, tx, s_rstride, lean);
}
// The same for the 32-value warp shapes (lengths 512 and 1024), at most 256
// threads: their registers would not fit more.
template <typename T, bool INL>
__global__ void __launch_bounds__(256) k_col_pass_wide(FftPlan p, int ncomp, C<T>* __restrict__ S, long long nspec,
                                                       const C<T>* __restrict__ khat, int hx, long long plane_stride,
                                                       long long pos_stride, int load_lim, int store_lim, int flags,
                                                       T inv_n, int tx, long long s_rstride, int lean) {
  col_pass_body<T, INL, true>(p, ncomp, S, nspec, khat, hx, plane_stride, pos_stride, load_lim, store_lim, flags,
                              inv_n, tx, s_rstride, lean);
}

// Column pass of a film (the y lines, with the K^ product between the forward
// and the inverse transform) for lengths A x A (64, 256) with the lines held
// in registers.  A CTA takes CR_TX kx columns; thread (t, b), t = threadIdx.x
// mod CR_TX, holds the values y = b + A a (a = 0 .. A-1) of the three
// components of column kx0 + t, loaded straight from the spectrum (CR_TX
// consecutive kx per row: whole sectors).  The forward transform is the
// arithmetic of fft_line_regs<T, false, A, A>: an A-point DFT over a in
// registers, the twiddles W^(b ka), a transpose among the A threads of the
// column through shared memory, an A-point DFT -- after which thread (t, b)
// holds the frequencies b + A kb, the layout the inverse starts from, so the
// K^ product and the inverse (fft_line_regs<T, true, A, A>'s arithmetic) run
// from the same registers and the results go straight back.  No line is
// staged in shared memory, and the transform, the product and the loads
// round exactly as in k_col_pass: the same results bit for bit, with about
// 40 % fewer instructions (ncu: 9.9 M against 17.0 M warp instructions for 32
// replicas of 256^2).  Holding three lines per thread takes 255 registers, so
// 2 CTAs of 128 threads fit per SM (12 % of the warp slots) and the loads'
// latency is exposed: at 256^2 it runs at k_col_pass's speed (32.2 against
// 33.0 us per batched sweep).  Capping it at 168 registers (3 CTAs) spilled
// and took 44.8 us; transforming one component at a time with the others
// parked in shared memory (126 registers) took 36.3 us.  It is an autotuner
// candidate (col_lean = 2).
constexpr int CR_TX = 8;  // kx columns per CTA
template <int A>
__host__ __device__ constexpr int col_reg_row() {
  return A * CR_TX + 8;  // transpose row (complex): conflict-free 8-byte accesses both ways
}
template <typename T, int A>
__host__ __device__ inline size_t col_reg_smem() {
  return ((size_t)A * A + 3 * (size_t)A * col_reg_row<A>()) * sizeof(C<T>);
}

// The three components' lines of column t: DFT over the thread's A values,
// twiddles, transpose (tb: three buffers of A rows), DFT.  first: the
// buffers are not being read by an earlier transform.
template <typename T, bool INV, int A>
__device__ __forceinline__ void col_reg_transform3(C<T> (&v)[3][A], C<T>* tb, const C<T>* roots, int t, int b,
                                                   bool first) {
  using V = C<T>;
  constexpr int RW = col_reg_row<A>();
#pragma unroll
  for (int c = 0; c < 3; ++c) RegDft<T, INV, A>::run(v[c]);
#pragma unroll
  for (int ka = 1; ka < A; ++ka) {
    const V w = roots[b * ka];
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c][ka] = INV ? cmulc(v[c][ka], w) : cmul(v[c][ka], w);
  }
  if (!first) __syncthreads();
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int ka = 0; ka < A; ++ka) tb[(c * A + ka) * RW + b * CR_TX + t] = v[c][ka];
  __syncthreads();
#pragma unroll
  for (int c = 0; c < 3; ++c) {
#pragma unroll
    for (int bb = 0; bb < A; ++bb) v[c][bb] = tb[(c * A + b) * RW + bb * CR_TX + t];
    RegDft<T, INV, A>::run(v[c]);
  }
}

template <typename T, int A>
__global__ void __launch_bounds__(CR_TX * A) k_col_reg(FftPlan p, C<T>* __restrict__ S, long long nspec,
                                                          const C<T>* __restrict__ khat, int hx, int pitch,
                                                          int load_lim, int store_lim, int flags, T inv_n,
                                                          long long s_rstride) {
  using V = C<T>;
  constexpr int L = A * A;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* roots = reinterpret_cast<V*>(smem_raw);  // exp(-2 pi i j / L), j < L
  V* tb = roots + L;
  S += blockIdx.z * s_rstride;
  const int t = threadIdx.x % CR_TX, b = threadIdx.x / CR_TX;
  const int kx = blockIdx.x * CR_TX + t;
  const bool ok = kx < hx;
  {
    const V* src = plan_tw<T>(p) + p.full_off;
    for (int i = threadIdx.x; i < L; i += blockDim.x) roots[i] = src[i];
  }
  pdl_wait();  // the spectrum is the x pass's output
  V v[3][A];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int a = 0; a < A; ++a) {
      const int row = b + A * a;
      v[c][a] = (ok && row < load_lim) ? S[c * nspec + (long long)row * pitch + kx] : cmk<V>(0, 0);
    }
  __syncthreads();  // roots
  col_reg_transform3<T, false, A>(v, tb, roots, t, b, true);
  // src/demag_cu.cu:98-111: real and imaginary parts of sum_b K_ab M_b, divided by N
#pragma unroll
  for (int kb = 0; kb < A; ++kb) {
    const int pos = b + A * kb;
    const V* kk = khat + (long long)pos * pitch + (ok ? kx : 0);
    V kxx = kk[0], kxy = kk[nspec], kxz = kk[2 * nspec];
    V kyy = kk[3 * nspec], kyz = kk[4 * nspec], kzz = kk[5 * nspec];
    if (flags & PASS_SYM) kxx.y = kxy.y = kxz.y = kyy.y = kyz.y = kzz.y = (T)0;
    const V mx = v[0][kb], my = v[1][kb], mz = v[2][kb];
    T hxr = (mx.x * kxx.x - mx.y * kxx.y) + (my.x * kxy.x - my.y * kxy.y) + (mz.x * kxz.x - mz.y * kxz.y);
    T hxi = (mx.x * kxx.y + mx.y * kxx.x) + (my.x * kxy.y + my.y * kxy.x) + (mz.x * kxz.y + mz.y * kxz.x);
    T hyr = (mx.x * kxy.x - mx.y * kxy.y) + (my.x * kyy.x - my.y * kyy.y) + (mz.x * kyz.x - mz.y * kyz.y);
    T hyi = (mx.x * kxy.y + mx.y * kxy.x) + (my.x * kyy.y + my.y * kyy.x) + (mz.x * kyz.y + mz.y * kyz.x);
    T hzr = (mx.x * kxz.x - mx.y * kxz.y) + (my.x * kyz.x - my.y * kyz.y) + (mz.x * kzz.x - mz.y * kzz.y);
    T hzi = (mx.x * kxz.y + mx.y * kxz.x) + (my.x * kyz.y + my.y * kyz.x) + (mz.x * kzz.y + mz.y * kzz.x);
    v[0][kb] = cmk<V>(hxr * inv_n, hxi * inv_n);
    v[1][kb] = cmk<V>(hyr * inv_n, hyi * inv_n);
    v[2][kb] = cmk<V>(hzr * inv_n, hzi * inv_n);
  }
  col_reg_transform3<T, true, A>(v, tb, roots, t, b, false);
  if (!ok) return;
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int kb = 0; kb < A; ++kb) {
      const int row = b + A * kb;
      if (row < store_lim) S[c * nspec + (long long)row * pitch + kx] = v[c][kb];
    }
}

// The same column pass with each component held by threads of its own:
// thread (c, t, b) of 3 CR_TX A holds component c of column t (k_col_reg's
// values y = b + A a).  Each component is transformed by exactly k_col_reg's
// arithmetic (col_reg_transform1, its own transpose buffer); for the K^
// product every thread writes its frequencies into its buffer in the
// transposes' layout and reads the other two components' from theirs, then
// forms its own component of sum_b K_ab M_b with k_col_reg's expressions.
// The results equal k_col_reg's (and k_col_pass's) bit for bit.  At 256^2
// (A = 16) it holds 168 registers per thread -- 12 warps per SM against
// k_col_reg's 8 -- and takes 30.3-31.1 us per batch of 32 replicas against
// 32.4; capped at 80 registers for two CTAs per SM it spilled and took 36.7,
// and 4 columns per CTA (192 threads, two CTAs per SM at 168 registers, less
// of the 129th column's tile wasted) took 30.6.  An autotuner candidate
// (col_lean = 3).
template <typename T, bool INV, int A>
__device__ __forceinline__ void col_reg_transform1(C<T> (&v)[A], C<T>* tb, const C<T>* roots, int t, int b,
                                                   bool first) {
  using V = C<T>;
  constexpr int RW = col_reg_row<A>();
  RegDft<T, INV, A>::run(v);
#pragma unroll
  for (int ka = 1; ka < A; ++ka) {
    const V w = roots[b * ka];
    v[ka] = INV ? cmulc(v[ka], w) : cmul(v[ka], w);
  }
  if (!first) __syncthreads();
#pragma unroll
  for (int ka = 0; ka < A; ++ka) tb[ka * RW + b * CR_TX + t] = v[ka];
  __syncthreads();
#pragma unroll
  for (int bb = 0; bb < A; ++bb) v[bb] = tb[b * RW + bb * CR_TX + t];
  RegDft<T, INV, A>::run(v);
}

template <typename T, int A>
__global__ void __launch_bounds__(3 * CR_TX * A)
    k_col_reg3(FftPlan p, C<T>* __restrict__ S, long long nspec, const C<T>* __restrict__ khat, int hx, int pitch,
               int load_lim, int store_lim, int flags, T inv_n, long long s_rstride) {
  using V = C<T>;
  constexpr int L = A * A, RW = col_reg_row<A>(), NT = CR_TX * A;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* roots = reinterpret_cast<V*>(smem_raw);  // exp(-2 pi i j / L), j < L
  V* tb = roots + L;                          // three buffers of A rows of RW
  S += blockIdx.z * s_rstride;
  const int c = threadIdx.x / NT, tt = threadIdx.x - c * NT;  // c is warp-uniform
  const int t = tt % CR_TX, b = tt / CR_TX;
  const int kx = blockIdx.x * CR_TX + t;
  const bool ok = kx < hx;
  {
    const V* src = plan_tw<T>(p) + p.full_off;
    for (int i = threadIdx.x; i < L; i += blockDim.x) roots[i] = src[i];
  }
  pdl_wait();  // the spectrum is the x pass's output
  V v[A];
#pragma unroll
  for (int a = 0; a < A; ++a) {
    const int row = b + A * a;
    v[a] = (ok && row < load_lim) ? S[c * nspec + (long long)row * pitch + kx] : cmk<V>(0, 0);
  }
  __syncthreads();  // roots
  V* tbc = tb + (size_t)c * A * RW;
  col_reg_transform1<T, false, A>(v, tbc, roots, t, b, true);
  __syncthreads();  // every thread has read its transpose
#pragma unroll
  for (int kb = 0; kb < A; ++kb) tbc[kb * RW + b * CR_TX + t] = v[kb];
  __syncthreads();
  // row c of K^: (xx, xy, xz), (xy, yy, yz) or (xz, yz, zz) in the six blocks
  // xx, xy, xz, yy, yz, zz
  const int o0 = c, o1 = c == 0 ? 1 : c == 1 ? 3 : 4, o2 = c == 0 ? 2 : c == 1 ? 4 : 5;
  // src/demag_cu.cu:98-111: real and imaginary parts of sum_b K_ab M_b, divided by N
#pragma unroll
  for (int kb = 0; kb < A; ++kb) {
    const int pos = b + A * kb;
    const V* kk = khat + (long long)pos * pitch + (ok ? kx : 0);
    V k0 = kk[o0 * nspec], k1 = kk[o1 * nspec], k2 = kk[o2 * nspec];
    if (flags & PASS_SYM) k0.y = k1.y = k2.y = (T)0;
    const int q = kb * RW + b * CR_TX + t;
    const V mx = tb[q], my = tb[A * RW + q], mz = tb[2 * A * RW + q];
    const T hr = (mx.x * k0.x - mx.y * k0.y) + (my.x * k1.x - my.y * k1.y) + (mz.x * k2.x - mz.y * k2.y);
    const T hi = (mx.x * k0.y + mx.y * k0.x) + (my.x * k1.y + my.y * k1.x) + (mz.x * k2.y + mz.y * k2.x);
    v[kb] = cmk<V>(hr * inv_n, hi * inv_n);
  }
  col_reg_transform1<T, true, A>(v, tbc, roots, t, b, false);
  if (!ok) return;
#pragma unroll
  for (int kb = 0; kb < A; ++kb) {
    const int row = b + A * kb;
    if (row < store_lim) S[c * nspec + (long long)row * pitch + kx] = v[kb];
  }
}

// Column pass for short lines (n <= 16: the padded z axis of thin 3-D
// lattices, short y axes): one thread per column (kx, plane) holding the three
// component lines in registers, transformed by ThreadDft -- no shared-memory
// staging, no barriers, and loads and stores coalesced across the threads'
// consecutive kx.  Same flags, product and tensor layout as k_col_pass.
template <typename T, int N>
__global__ void __launch_bounds__(128) k_col_short(FftPlan p, C<T>* __restrict__ S, long long nspec,
                                                   const C<T>* __restrict__ khat, int hx, long long plane_stride,
                                                   long long pos_stride, int load_lim, int store_lim, int flags,
                                                   T inv_n, long long s_rstride) {
  using V = C<T>;
  __shared__ V rt[N];
  S += blockIdx.z * s_rstride;
  {
    const V* src = plan_tw<T>(p) + p.full_off;
    for (int i = threadIdx.x; i < N; i += blockDim.x) rt[i] = src[i];
  }
  pdl_wait();
  __syncthreads();
  const int kx = blockIdx.x * blockDim.x + threadIdx.x;
  if (kx >= hx) return;
  const long long base = (long long)blockIdx.y * plane_stride + kx;
  V v[3][N];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int z = 0; z < N; ++z) v[c][z] = z < load_lim ? S[c * nspec + base + z * pos_stride] : cmk<V>(0, 0);
  if (flags & PASS_FWD) {
#pragma unroll
    for (int c = 0; c < 3; ++c) ThreadDft<T, false, N, 1>::run(v[c], rt);
  }
  if (flags & PASS_MUL) {
#pragma unroll
    for (int z = 0; z < N; ++z) {
      const V* kk = khat + base + z * pos_stride;
      V kxx = kk[0], kxy = kk[nspec], kxz = kk[2 * nspec];
      V kyy = kk[3 * nspec], kyz = kk[4 * nspec], kzz = kk[5 * nspec];
      if (flags & PASS_SYM) kxx.y = kxy.y = kxz.y = kyy.y = kyz.y = kzz.y = (T)0;
      const V mx = v[0][z], my = v[1][z], mz = v[2][z];
      T hxr = (mx.x * kxx.x - mx.y * kxx.y) + (my.x * kxy.x - my.y * kxy.y) + (mz.x * kxz.x - mz.y * kxz.y);
      T hxi = (mx.x * kxx.y + mx.y * kxx.x) + (my.x * kxy.y + my.y * kxy.x) + (mz.x * kxz.y + mz.y * kxz.x);
      T hyr = (mx.x * kxy.x - mx.y * kxy.y) + (my.x * kyy.x - my.y * kyy.y) + (mz.x * kyz.x - mz.y * kyz.y);
      T hyi = (mx.x * kxy.y + mx.y * kxy.x) + (my.x * kyy.y + my.y * kyy.x) + (mz.x * kyz.y + mz.y * kyz.x);
      T hzr = (mx.x * kxz.x - mx.y * kxz.y) + (my.x * kyz.x - my.y * kyz.y) + (mz.x * kzz.x - mz.y * kzz.y);
      T hzi = (mx.x * kxz.y + mx.y * kxz.x) + (my.x * kyz.y + my.y * kyz.x) + (mz.x * kzz.y + mz.y * kzz.x);
      v[0][z] = cmk<V>(hxr * inv_n, hxi * inv_n);
      v[1][z] = cmk<V>(hyr * inv_n, hyi * inv_n);
      v[2][z] = cmk<V>(hzr * inv_n, hzi * inv_n);
    }
  }
  if (flags & PASS_INV) {
#pragma unroll
    for (int c = 0; c < 3; ++c) ThreadDft<T, true, N, 1>::run(v[c], rt);
  }
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int z = 0; z < N; ++z)
      if (z < store_lim) S[c * nspec + base + z * pos_stride] = v[c][z];
}

// The short-line kernel for length n, or null.
template <typename T>
using ColShortFn = void (*)(FftPlan, C<T>*, long long, const C<T>*, int, long long, long long, int, int, int, T,
                            long long);
template <typename T>
ColShortFn<T> col_short_kernel(int n) {
  switch (n) {
#define MMC_CS(N_) \
  case N_:         \
    return k_col_short<T, N_>;
    MMC_CS(2) MMC_CS(3) MMC_CS(4) MMC_CS(5) MMC_CS(6) MMC_CS(7) MMC_CS(8) MMC_CS(9) MMC_CS(10) MMC_CS(11)
    MMC_CS(12) MMC_CS(13) MMC_CS(14) MMC_CS(15) MMC_CS(16)
#undef MMC_CS
    default:
      return nullptr;
  }
}

// =========================================================== lattice helpers
// Neighbour index along an axis, or -1 when the bond does not exist (open
// edge, or a periodic axis of length 1 where the neighbour is the cell itself).
__device__ __forceinline__ long long nbr_idx(const Geom& g, int x, int y, int z, int axis, int dir) {
  int c[3] = {x, y, z};
  const int n[3] = {g.nx, g.ny, g.nz};
  int v = c[axis] + dir;
  if (v < 0 || v >= n[axis]) {
    if (!g.per[axis]) return -1;
    v = v < 0 ? v + n[axis] : v - n[axis];
  }
  if (v == c[axis]) return -1;
  c[axis] = v;
  return c[0] + (long long)g.nx * (c[1] + (long long)g.ny * c[2]);
}

// nbr_idx from the cell's own index i: a step of +-stride, wrapped on a
// periodic axis; the same result without rebuilding the index.
__device__ __forceinline__ long long nbr_step(const Geom& g, long long i, int x, int y, int z, int axis, int dir) {
  const int n = axis == 0 ? g.nx : axis == 1 ? g.ny : g.nz;
  const int c = axis == 0 ? x : axis == 1 ? y : z;
  const long long stride = axis == 0 ? 1 : axis == 1 ? (long long)g.nx : (long long)g.nx * g.ny;
  const int v = c + dir;
  long long j = i + dir * stride;
  if (v < 0 || v >= n) {
    if (!g.per[axis]) return -1;
    j += v < 0 ? n * stride : -n * stride;
  }
  return n == 1 ? -1 : j;  // a periodic axis of length 1 wraps onto the cell itself
}

__device__ __forceinline__ int axis_color(int v, int n, int per) {
  if (per && (n & 1) && n > 1 && v == n - 1) return 2;
  return v & 1;
}

__device__ __forceinline__ int cell_color(const Geom& g, int x, int y, int z) {
  int s = axis_color(x, g.nx, g.per[0]) + axis_color(y, g.ny, g.per[1]) + axis_color(z, g.nz, g.per[2]);
  return g.ncolors == 2 ? (s & 1) : (s % 3);
}

// =========================================================== Metropolis sweep
//
// One sublattice colour of one sweep.  This replaces mcKernel2
// (src/mc_sampling.h:27-41, launched src/main.cu:1101-1120), whose body is not
// published.  Cells of one colour share no exchange or DMI bond, so they are
// updated in place concurrently.  For cell i:
//   F   = sum_a wex_a sum_(+-) m_nbr + DMI(nbr) + cz + cd (h_i - K0 m_i)
//   dE  = -(m' - m).F - can[(m'.u)^2 - (m.u)^2] - cd/2 [m'K0m' - mK0m]   (units of kT)
//   accept when dE <= 0 or u < exp(-dE)
// with (u0, u1, u) = Philox4x32-10(key = seed; counter = (i, sweep, stage, 0)),
// m' = (sqrt(1-z^2) cos 2 pi u1, sqrt(1-z^2) sin 2 pi u1, z = 2 u0 - 1).
template <typename T>
struct Prop;

template <>
struct Prop<double> {
  __device__ static void draw(mmcm::u32x4 r, double& px, double& py, double& pz, double& ua) {
    pz = 2.0 * mmcm::u01_f64(r.x) - 1.0;
    double t = 1.0 - pz * pz;
    if (t < 0) t = 0;
    double s = mmcm::dsqrt(t), sn, cs;
    mmcm::sincospi(2.0 * mmcm::u01_f64(r.y), &sn, &cs);
    px = s * cs;
    py = s * sn;
    ua = mmcm::u01_f64(r.z);
  }
  __device__ static bool accept(double dE, double ua) { return dE <= 0.0 || ua < mmcm::exp(-dE); }
};

template <>
struct Prop<float> {
  // FP32: the hardware sine and cosine of phi - pi in (-pi, pi), where their
  // absolute error is about 4e-7, negated (exact), and sqrt(t) as t / sqrt(t)
  // from the hardware reciprocal square root; t = 1 - z^2 >= 2^-22 because
  // u01_f32 never returns 0 or 1.
  __device__ static void draw(mmcm::u32x4 r, float& px, float& py, float& pz, float& ua) {
    pz = 2.0f * mmcm::u01_f32(r.x) - 1.0f;
    const float t = 1.0f - pz * pz;
    const float s = t * rsqrtf(t);
    float sn, cs;
    __sincosf(6.28318530717958647692f * mmcm::u01_f32(r.y) - 3.14159265358979323846f, &sn, &cs);
    px = -(s * cs);
    py = -(s * sn);
    ua = mmcm::u01_f32(r.z);
  }
  __device__ static bool accept(float dE, float ua) { return dE <= 0.0f || ua < __expf(-dE); }
};

// Neighbour values of one trial: v[a][s] is the neighbour along axis a on side
// s (0 = -, 1 = +); has[a][s] tells whether that bond exists.
template <typename T>
struct Nbrs {
  T v[3][2][3];
  bool has[3][2];
};

// Proposal of one trial: Philox4x32-10(key = seed; counter = (cell, sweep,
// stage, 0)) -> direction m' and acceptance uniform ua.
template <typename T>
struct Proposal {
  T x, y, z, ua;
};

template <typename T>
__device__ __forceinline__ Proposal<T> mc_propose(const McCoef<T>& c, uint32_t cell, uint32_t stage, uint32_t sweep) {
  mmcm::u32x4 ctr = {cell, sweep, stage, mmcm::STREAM_SWEEP};
  mmcm::u32x4 r = mmcm::philox4x32_10(ctr, c.key0, c.key1);
  Proposal<T> p;
  Prop<T>::draw(r, p.x, p.y, p.z, p.ua);
  return p;
}

// The Metropolis decision for one cell from its neighbour values, its own m,
// its demag field h and its proposal.  Shared by every sweep kernel so that
// all paths round identically.
template <typename T>
__device__ __forceinline__ bool mc_accept(const McCoef<T>& c, const Nbrs<T>& nb, T ox, T oy, T oz, T hx, T hy, T hz,
                                          const Proposal<T>& p) {
  T Fx = 0, Fy = 0, Fz = 0;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      if (!nb.has[a][s]) continue;
      Fx = Fx + c.wex[a] * nb.v[a][s][0];
      Fy = Fy + c.wex[a] * nb.v[a][s][1];
      Fz = Fz + c.wex[a] * nb.v[a][s][2];
    }
  const T dxmz = (nb.has[0][1] ? nb.v[0][1][2] : (T)0) - (nb.has[0][0] ? nb.v[0][0][2] : (T)0);
  const T dxmx = (nb.has[0][1] ? nb.v[0][1][0] : (T)0) - (nb.has[0][0] ? nb.v[0][0][0] : (T)0);
  const T dymz = (nb.has[1][1] ? nb.v[1][1][2] : (T)0) - (nb.has[1][0] ? nb.v[1][0][2] : (T)0);
  const T dymy = (nb.has[1][1] ? nb.v[1][1][1] : (T)0) - (nb.has[1][0] ? nb.v[1][0][1] : (T)0);
  Fx = Fx + c.wdm[0] * dxmz;
  Fy = Fy + c.wdm[1] * dymz;
  Fz = Fz - (c.wdm[0] * dxmx + c.wdm[1] * dymy);
  Fx = Fx + c.cz[0];
  Fy = Fy + c.cz[1];
  Fz = Fz + c.cz[2];
  if constexpr (sizeof(T) == 4) {
    // FP32: the same energy difference regrouped with d = m' - m, s = m' + m
    // and K0 symmetric,
    //   dE = -d . [F_local + cd h + (cd / 2) K0 d + can (s . u) u],
    // where F_local is the exchange, DMI and Zeeman part of F: the terms in
    // K0 m cancel, and the quadratic forms need no difference of squares.
    const T ddx = p.x - ox, ddy = p.y - oy, ddz = p.z - oz;
    if (c.cd != (T)0) {
      Fx = Fx + c.cd * hx + (c.k0h[0] * ddx + c.k0h[1] * ddy + c.k0h[2] * ddz);
      Fy = Fy + c.cd * hy + (c.k0h[1] * ddx + c.k0h[3] * ddy + c.k0h[4] * ddz);
      Fz = Fz + c.cd * hz + (c.k0h[2] * ddx + c.k0h[4] * ddy + c.k0h[5] * ddz);
    }
    const T su = (p.x + ox) * c.u[0] + (p.y + oy) * c.u[1] + (p.z + oz) * c.u[2];
    const T cs = c.can * su;
    Fx = Fx + cs * c.u[0];
    Fy = Fy + cs * c.u[1];
    Fz = Fz + cs * c.u[2];
    return Prop<T>::accept(-(ddx * Fx + ddy * Fy + ddz * Fz), p.ua);
  }
  if (c.cd != (T)0) {
    const T sx = c.k0[0] * ox + c.k0[1] * oy + c.k0[2] * oz;
    const T sy = c.k0[1] * ox + c.k0[3] * oy + c.k0[4] * oz;
    const T sz = c.k0[2] * ox + c.k0[4] * oy + c.k0[5] * oz;
    Fx = Fx + c.cd * (hx - sx);
    Fy = Fy + c.cd * (hy - sy);
    Fz = Fz + c.cd * (hz - sz);
  }
  const T px = p.x, py = p.y, pz = p.z;
  const T ddx = px - ox, ddy = py - oy, ddz = pz - oz;
  T dE = -(ddx * Fx + ddy * Fy + ddz * Fz);
  const T pun = px * c.u[0] + py * c.u[1] + pz * c.u[2];
  const T puo = ox * c.u[0] + oy * c.u[1] + oz * c.u[2];
  dE = dE - c.can * (pun * pun - puo * puo);
  if (c.cd != (T)0) {
    const T qn = px * (c.k0[0] * px + c.k0[1] * py + c.k0[2] * pz) + py * (c.k0[1] * px + c.k0[3] * py + c.k0[4] * pz) +
                 pz * (c.k0[2] * px + c.k0[4] * py + c.k0[5] * pz);
    const T qo = ox * (c.k0[0] * ox + c.k0[1] * oy + c.k0[2] * oz) + oy * (c.k0[1] * ox + c.k0[3] * oy + c.k0[4] * oz) +
                 oz * (c.k0[2] * ox + c.k0[4] * oy + c.k0[5] * oz);
    dE = dE - (T)0.5 * c.cd * (qn - qo);
  }
  return Prop<T>::accept(dE, p.ua);
}

template <typename T>
__device__ __forceinline__ bool mc_decide(const McCoef<T>& c, const Nbrs<T>& nb, T ox, T oy, T oz, T hx, T hy, T hz,
                                          uint32_t cell, uint32_t stage, uint32_t sweep, T& px, T& py, T& pz) {
  const Proposal<T> p = mc_propose<T>(c, cell, stage, sweep);
  px = p.x;
  py = p.y;
  pz = p.z;
  return mc_accept<T>(c, nb, ox, oy, oz, hx, hy, hz, p);
}

template <typename T>
__device__ __forceinline__ bool mc_trial(const Geom& g, const McCoef<T>& c, T* __restrict__ m,
                                         const T* __restrict__ h, uint32_t stage, uint32_t sweep, int x, int y,
                                         int z) {
  const long long n = g.n;
  T* mx = m;
  T* my = m + n;
  T* mz = m + 2 * n;
  const long long i = x + (long long)g.nx * (y + (long long)g.ny * z);
  const T ox = mx[i], oy = my[i], oz = mz[i];
  Nbrs<T> nb;
  const bool film = g.nz == 1;  // no z bonds: skip their index work and loads
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      if (a == 2 && film) {
        nb.has[a][s] = false;
        nb.v[a][s][0] = ox;
        nb.v[a][s][1] = oy;
        nb.v[a][s][2] = oz;
        continue;
      }
      const long long j = nbr_step(g, i, x, y, z, a, s ? 1 : -1);
      nb.has[a][s] = j >= 0;
      const long long jj = j >= 0 ? j : i;
      nb.v[a][s][0] = mx[jj];
      nb.v[a][s][1] = my[jj];
      nb.v[a][s][2] = mz[jj];
    }
  T hx = 0, hy = 0, hz = 0;
  if (c.cd != (T)0) {
    hx = h[i];
    hy = h[n + i];
    hz = h[2 * n + i];
  }
  T px, py, pz;
  if (mc_decide<T>(c, nb, ox, oy, oz, hx, hy, hz, (uint32_t)i, stage, sweep, px, py, pz)) {
    mx[i] = px;
    my[i] = py;
    mz[i] = pz;
    return true;
  }
  return false;
}

__device__ __forceinline__ void count_accepts(bool acc, unsigned long long* counter) {
  const unsigned mask = __ballot_sync(0xffffffffu, acc);
  if ((threadIdx.x & 31) == 0 && mask) atomicAdd(counter, (unsigned long long)__popc(mask));
}

// Two-colour checkerboard: thread t -> row t / hxc, x = 2 (t mod hxc) + parity.
template <typename T>
__global__ void __launch_bounds__(256, 4) k_mc_checker(Geom g, const McCoef<T>* __restrict__ cp, T* __restrict__ m, const T* __restrict__ h,
                             const SweepCounters* __restrict__ ctr, int color, unsigned long long* acc) {
  pdl_wait();
  // replica blockIdx.z of a batch: its own coefficients, state and counter
  const McCoef<T> c = cp[blockIdx.z];
  m += blockIdx.z * 3 * g.n;
  h += blockIdx.z * 3 * g.n;
  acc += blockIdx.z;
  const int hxc = (g.nx + 1) >> 1;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nrows = (long long)g.ny * g.nz;
  bool accepted = false;
  if (t < nrows * hxc) {
    const int row = g.dhxc.div((int)t);
    const int j = (int)t - row * hxc;
    const int z = g.dny.div(row), y = row - z * g.ny;
    const int x = 2 * j + ((color + y + z) & 1);
    if (x < g.nx) accepted = mc_trial<T>(g, c, m, h, ctr->stage, ctr->sweep, x, y, z);
  }
  count_accepts(accepted, acc);
}

// General colouring (odd periodic axes): every thread tests its cell's colour.
template <typename T>
__global__ void __launch_bounds__(256, 4) k_mc_general(Geom g, const McCoef<T>* __restrict__ cp, T* __restrict__ m, const T* __restrict__ h,
                             const SweepCounters* __restrict__ ctr, int color, unsigned long long* acc) {
  const McCoef<T> c = cp[blockIdx.z];
  m += blockIdx.z * 3 * g.n;
  h += blockIdx.z * 3 * g.n;
  acc += blockIdx.z;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  bool accepted = false;
  if (i < g.n) {
    const int x = (int)(i % g.nx), y = (int)((i / g.nx) % g.ny), z = (int)(i / ((long long)g.nx * g.ny));
    if (cell_color(g, x, y, z) == color) accepted = mc_trial<T>(g, c, m, h, ctr->stage, ctr->sweep, x, y, z);
  }
  count_accepts(accepted, acc);
}

// One colour of a two-colour film sweep (nz = 1, nx a multiple of 4) with
// 16-byte loads: a thread owns a segment of 4 consecutive cells of one row
// and makes the decisions of its 2 cells of this colour.  The row segment, the
// same segment of the rows above and below, and one cell on each side are
// loaded as whole vectors; the segment is stored back whole (its cells of the
// other colour are written with the values just read, which no thread of this
// launch changes).  Decisions are those of k_mc_checker (same mc_accept, same
// inputs).
template <typename T>
struct Vec4 {
  T v[4];
};
template <typename T>
__device__ __forceinline__ Vec4<T> ld4(const T* p) {
  Vec4<T> r;
  if constexpr (sizeof(T) == 4) {
    const float4 a = *reinterpret_cast<const float4*>(p);
    r.v[0] = a.x, r.v[1] = a.y, r.v[2] = a.z, r.v[3] = a.w;
  } else {
    const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
    r.v[0] = a.x, r.v[1] = a.y, r.v[2] = b.x, r.v[3] = b.y;
  }
  return r;
}
template <typename T>
__device__ __forceinline__ void st4(T* p, const Vec4<T>& r) {
  if constexpr (sizeof(T) == 4) {
    *reinterpret_cast<float4*>(p) = make_float4(r.v[0], r.v[1], r.v[2], r.v[3]);
  } else {
    reinterpret_cast<double2*>(p)[0] = make_double2(r.v[0], r.v[1]);
    reinterpret_cast<double2*>(p)[1] = make_double2(r.v[2], r.v[3]);
  }
}

// The decisions of the two cells at offsets P0 and P0 + 2 of a segment.
// ALLB: every x and y bond exists (both axes periodic, ny > 1), so the
// availability flags are compile-time true.  Z3: a 3-D lattice, with the
// segments of the layers below (zd) and above (zu) and their flags; films
// pass anything there.
template <typename T, int P0, bool ALLB, bool Z3 = false>
__device__ __forceinline__ bool quad_cells(const McCoef<T>& c, Vec4<T> (&own)[3], const Vec4<T> (&up)[3],
                                           const Vec4<T> (&dn)[3], const T (&lft)[3], const T (&rgt)[3],
                                           const Vec4<T> (&hh)[3], bool hl, bool hr, bool hd, bool hu,
                                           uint32_t cell0, uint32_t stage, uint32_t sweep, unsigned int& mine,
                                           const Vec4<T> (&zd)[3], const Vec4<T> (&zu)[3], bool hzd, bool hzu) {
  if constexpr (ALLB) hl = hr = hd = hu = true;
  if constexpr (!Z3) hzd = hzu = false;
  bool changed = false;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int o = P0 + 2 * q;  // compile-time after unrolling
    Nbrs<T> nb;
    const bool lin = o > 0, rin = o < 3;
    nb.has[0][0] = lin || hl;
    nb.has[0][1] = rin || hr;
    nb.has[1][0] = hd;
    nb.has[1][1] = hu;
    nb.has[2][0] = hzd;
    nb.has[2][1] = hzu;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const T ov = own[k].v[o];
      nb.v[0][0][k] = lin ? own[k].v[(o + 3) & 3] : (hl ? lft[k] : ov);
      nb.v[0][1][k] = rin ? own[k].v[(o + 1) & 3] : (hr ? rgt[k] : ov);
      nb.v[1][0][k] = hd ? dn[k].v[o] : ov;
      nb.v[1][1][k] = hu ? up[k].v[o] : ov;
      nb.v[2][0][k] = hzd ? zd[k].v[o] : ov;
      nb.v[2][1][k] = hzu ? zu[k].v[o] : ov;
    }
    const Proposal<T> pr = mc_propose<T>(c, cell0 + (uint32_t)o, stage, sweep);
    if (mc_accept<T>(c, nb, own[0].v[o], own[1].v[o], own[2].v[o], hh[0].v[o], hh[1].v[o], hh[2].v[o], pr)) {
      own[0].v[o] = pr.x;
      own[1].v[o] = pr.y;
      own[2].v[o] = pr.z;
      changed = true;
      ++mine;
    }
  }
  return changed;
}

__host__ __device__ inline bool mc_quad_ok(const Geom& g) { return g.ncolors == 2 && g.nx % 4 == 0; }
// every x and y bond of a film exists
__host__ __device__ inline bool mc_all_bonds(const Geom& g) { return g.per[0] && g.per[1] && g.nx > 1 && g.ny > 1; }
// the staged form (k_mc_band) for the same lattices, up to 1024 cells per row
// (a band of one row then fits in 96 KB of shared memory in FP64)
constexpr size_t MC_BAND_SMEM_MAX = 96 * 1024;
__host__ __device__ inline bool mc_band_ok(const Geom& g) { return g.nz == 1 && mc_quad_ok(g) && g.nx <= 1024; }

// Z3: 3-D lattices (nz > 1), with the segments of the layers below and above.
template <typename T, bool ALLB, bool Z3>
__global__ void __launch_bounds__(256) k_mc_quad(Geom g, const McCoef<T>* __restrict__ cp, T* __restrict__ m,
                                                 const T* __restrict__ h, const SweepCounters* __restrict__ ctr,
                                                 int color, unsigned long long* acc) {
  pdl_wait();
  const McCoef<T> c = cp[blockIdx.z];
  const long long n = g.n;
  m += blockIdx.z * 3 * n;
  h += blockIdx.z * 3 * n;
  acc += blockIdx.z;
  const int nseg = g.nx >> 2;
  // two segments per thread, a grid-stride apart: the coefficients and the
  // set-up are shared by both, and the second segment's loads overlap the
  // first one's work (measured 4 us faster per batched sweep than one segment)
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
  const int tstride = gridDim.x * blockDim.x;
  unsigned int mine = 0;
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int t = t0 + u * tstride;
    if (t < nseg * g.ny * g.nz) {
      // t / (nx / 4) == (4 t) / nx: the multiply-shift divider by nx, no run-time division
      const int row = g.dnx.div(4 * t), s = t - row * nseg;
      int z = 0, y = row;
      if constexpr (Z3) {
        z = g.dny.div(row);
        y = row - z * g.ny;
      }
      const int x0 = 4 * s;
      const long long rowb = (long long)row * g.nx;
      const long long plane = (long long)g.nx * g.ny;
      // neighbour rows: wrapped on a periodic axis, missing at an open edge or
      // when the axis has length 1
      int yu = y + 1, yd = y - 1;
      bool hu = true, hd = true;
      if (yu >= g.ny) { if (g.per[1]) yu -= g.ny; else hu = false; }
      if (yd < 0) { if (g.per[1]) yd += g.ny; else hd = false; }
      if (g.ny == 1) hu = hd = false;
      int zu = z + 1, zd = z - 1;
      bool hzu = Z3, hzd = Z3;
      if constexpr (Z3) {
        if (zu >= g.nz) { if (g.per[2]) zu -= g.nz; else hzu = false; }
        if (zd < 0) { if (g.per[2]) zd += g.nz; else hzd = false; }
      }
      // side cells
      int xl = x0 - 1, xr = x0 + 4;
      bool hl = true, hr = true;
      if (xl < 0) { if (g.per[0]) xl += g.nx; else hl = false; }
      if (xr >= g.nx) { if (g.per[0]) xr -= g.nx; else hr = false; }
      if constexpr (ALLB) hu = hd = hl = hr = true;
      // this colour's cells sit at offsets p0 and p0 + 2 (x0 is even), so only
      // one side cell is a neighbour: the left one for p0 = 0, the right one
      // for p0 = 1
      const int p0 = (color + y + z) & 1;
      const long long zbase = (long long)z * plane;
      Vec4<T> own[3], up[3], dn[3], zup[3], zdn[3];
      T lft[3], rgt[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const T* base = m + k * n;
        own[k] = ld4<T>(base + rowb + x0);
        up[k] = hu ? ld4<T>(base + zbase + (long long)yu * g.nx + x0) : own[k];
        dn[k] = hd ? ld4<T>(base + zbase + (long long)yd * g.nx + x0) : own[k];
        if constexpr (Z3) {
          zup[k] = hzu ? ld4<T>(base + (long long)zu * plane + (long long)y * g.nx + x0) : own[k];
          zdn[k] = hzd ? ld4<T>(base + (long long)zd * plane + (long long)y * g.nx + x0) : own[k];
        } else {
          zup[k] = zdn[k] = own[k];
        }
        lft[k] = (hl && p0 == 0) ? base[rowb + xl] : (T)0;
        rgt[k] = (hr && p0 == 1) ? base[rowb + xr] : (T)0;
      }
      Vec4<T> hh[3];
      const bool dm = c.cd != (T)0;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (dm) hh[k] = ld4<T>(h + k * n + rowb + x0);
        else hh[k].v[0] = hh[k].v[1] = hh[k].v[2] = hh[k].v[3] = (T)0;
      }
      // the offsets are compile-time inside quad_cells so the vectors stay in
      // registers
      bool changed;
      if (p0 == 0)
        changed = quad_cells<T, 0, ALLB, Z3>(c, own, up, dn, lft, rgt, hh, hl, hr, hd, hu, (uint32_t)(rowb + x0),
                                             ctr->stage, ctr->sweep, mine, zdn, zup, hzd, hzu);
      else
        changed = quad_cells<T, 1, ALLB, Z3>(c, own, up, dn, lft, rgt, hh, hl, hr, hd, hu, (uint32_t)(rowb + x0),
                                             ctr->stage, ctr->sweep, mine, zdn, zup, hzd, hzu);
      if (changed) {
#pragma unroll
        for (int k = 0; k < 3; ++k) st4<T>(m + k * n + rowb + x0, own[k]);
      }
    }
  }
  unsigned int v = mine;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(acc, (unsigned long long)v);
}

// One colour of a two-colour film sweep (the k_mc_quad film cases) with the rows
// a CTA needs staged in shared memory first: the CTA owns a band of `band`
// rows of one replica, copies m rows y0-1 .. y0+band (wrapped on a periodic
// axis) and h rows y0 .. y0+band-1 with 16-byte asynchronous copies, which
// hold no registers while they land, and then runs k_mc_quad's per-thread
// work (4-cell segments, the same quad_cells) from shared memory.  Fewer
// registers per thread than k_mc_quad, whose vector loads all sit in
// registers at once, so more warps per SM hide the copies' latency.
// Shared memory: (band + 2) x 3 rows of m and band x 3 rows of h.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

template <typename T>
__host__ __device__ inline size_t mc_band_smem(const Geom& g, int band) {
  return (size_t)(2 * band + 2) * 3 * g.nx * sizeof(T);
}
// rows per CTA: about one 4-cell segment per thread
template <typename T>
inline int mc_band_rows(const Geom& g, int threads) {
  int band = std::max(1, std::min(g.ny, 4 * threads / g.nx));
  while (band > 1 && mc_band_smem<T>(g, band) > MC_BAND_SMEM_MAX) band /= 2;
  return band;
}

// The decisions of this colour on rows y0 .. y0+nb-1 of one replica from rows
// staged in shared memory -- ms[slot][comp][x] with slot s = row y0-1+s, hs
// [row][comp][x] (read when dm) -- the CTA's threads striding over the rows'
// 4-cell segments (k_mc_quad's per-thread work, the same quad_cells); the
// segments that changed are stored to m (this replica's), and accepts are
// added to mine.
template <typename T, bool ALLB>
__device__ __forceinline__ void band_segments(const Geom& g, const McCoef<T>& c, const T* ms, const T* hs,
                                              T* __restrict__ m, int y0, int nb, int color, bool dm,
                                              const FastDiv& dseg, uint32_t stage, uint32_t sweep,
                                              unsigned int& mine) {
  const int nx = g.nx, ny = g.ny;
  const long long n = g.n;
  const int nseg = (int)dseg.d;
  for (int t = threadIdx.x; t < nb * nseg; t += blockDim.x) {
    const int rr = dseg.div(t), s = t - rr * nseg;
    const int y = y0 + rr;
    const int x0 = 4 * s;
    bool hu = true, hd = true;
    if (y + 1 >= ny && !g.per[1]) hu = false;
    if (y - 1 < 0 && !g.per[1]) hd = false;
    if (ny == 1) hu = hd = false;
    int xl = x0 - 1, xr = x0 + 4;
    bool hl = true, hr = true;
    if (xl < 0) { if (g.per[0]) xl += nx; else hl = false; }
    if (xr >= nx) { if (g.per[0]) xr -= nx; else hr = false; }
    if constexpr (ALLB) hu = hd = hl = hr = true;
    const int p0 = (color + y) & 1;
    const T* own_r = ms + (size_t)(rr + 1) * 3 * nx;
    const T* up_r = own_r + 3 * nx;
    const T* dn_r = own_r - 3 * nx;
    Vec4<T> own[3], up[3], dn[3], hh[3];
    T lft[3], rgt[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      own[k] = ld4<T>(own_r + k * nx + x0);
      up[k] = hu ? ld4<T>(up_r + k * nx + x0) : own[k];
      dn[k] = hd ? ld4<T>(dn_r + k * nx + x0) : own[k];
      lft[k] = (hl && p0 == 0) ? own_r[k * nx + xl] : (T)0;
      rgt[k] = (hr && p0 == 1) ? own_r[k * nx + xr] : (T)0;
      if (dm) hh[k] = ld4<T>(hs + ((size_t)rr * 3 + k) * nx + x0);
      else hh[k].v[0] = hh[k].v[1] = hh[k].v[2] = hh[k].v[3] = (T)0;
    }
    const long long rowb = (long long)y * nx;
    bool changed;
    if (p0 == 0)
      changed = quad_cells<T, 0, ALLB>(c, own, up, dn, lft, rgt, hh, hl, hr, hd, hu, (uint32_t)(rowb + x0), stage,
                                       sweep, mine, own, own, false, false);
    else
      changed = quad_cells<T, 1, ALLB>(c, own, up, dn, lft, rgt, hh, hl, hr, hd, hu, (uint32_t)(rowb + x0), stage,
                                       sweep, mine, own, own, false, false);
    if (changed) {
#pragma unroll
      for (int k = 0; k < 3; ++k) st4<T>(m + k * n + rowb + x0, own[k]);
    }
  }
}

// (Three CTAs of 256 threads per SM in FP32 -- 80 registers, a few spilled
// -- and two in FP64.)
template <typename T, bool ALLB>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 2) k_mc_band(Geom g, const McCoef<T>* __restrict__ cp, T* __restrict__ m,
                                                    const T* __restrict__ h, const SweepCounters* __restrict__ ctr,
                                                    int color, int band, FastDiv dchunk, FastDiv dseg,
                                                    unsigned long long* acc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nx = g.nx, ny = g.ny;
  const long long n = g.n;
  T* ms = reinterpret_cast<T*>(smem_raw);  // [slot][comp][x], slot s = row y0 - 1 + s
  T* hs = ms + (size_t)(band + 2) * 3 * nx;  // [row][comp][x]
  const McCoef<T> c = cp[blockIdx.z];
  m += blockIdx.z * 3 * n;
  h += blockIdx.z * 3 * n;
  acc += blockIdx.z;
  const int y0 = blockIdx.x * band;
  const int nb = min(band, ny - y0);
  const bool dm = c.cd != (T)0;
  const int per = (int)dchunk.d;  // 16-byte chunks per row
  constexpr int E = 16 / (int)sizeof(T);
  const int nm = (nb + 2) * 3 * per, nh = dm ? nb * 3 * per : 0;
  for (int i = threadIdx.x; i < nm + nh; i += blockDim.x) {
    const bool isM = i < nm;
    const int j = isM ? i : i - nm;
    const int row = dchunk.div(j), q = j - row * per;  // row = slot * 3 + comp (m) or r * 3 + comp (h)
    const int slot = row / 3, comp = row - slot * 3;
    if (isM) {
      int y = y0 - 1 + slot;
      if (y < 0 || y >= ny) {
        if (!g.per[1] || ny == 1) continue;
        y = y < 0 ? y + ny : y - ny;
      }
      cp_async16(ms + (size_t)row * nx + q * E, m + comp * n + (long long)y * nx + q * E);
    } else {
      cp_async16(hs + (size_t)row * nx + q * E, h + comp * n + (long long)(y0 + slot) * nx + q * E);
    }
  }
  cp_async_wait_all();
  __syncthreads();
  unsigned int mine = 0;
  band_segments<T, ALLB>(g, c, ms, hs, m, y0, nb, color, dm, dseg, ctr->stage, ctr->sweep, mine);
  unsigned int v = mine;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(acc, (unsigned long long)v);
}

// ---------------------------------------------- pipelined staged Metropolis
// One colour of a two-colour film sweep (the k_mc_band lattices) by
// persistent CTAs.  Work items are (replica, band of rows); CTA b takes the
// items [b chunk, (b + 1) chunk), consecutive bands of one replica, so its
// coefficients change rarely.  A band's rows -- m rows y0-1 .. y0+nb (wrapped
// on a periodic axis) and h rows y0 .. y0+nb-1, whole rows of one component
// each -- are fetched by bulk asynchronous copies (cp.async.bulk, the TMA
// engine) into one of nst (2-4) shared-memory buffers, their completion
// counted by that buffer's mbarrier (transaction bytes).  Warp 0 issues the
// copies of item i + nst as soon as item i's buffer is free (after the CTA
// barrier that ends item i), so the loads of later bands land while the CTA
// decides the current ones: no registers or issue slots spent on copying, and
// none of the load latency on the decisions' critical path.  Every warp waits
// on its buffer's mbarrier itself, so no warp waits for the producer's
// issuing; the producer reads the next item's replica flag (demag on or off)
// before the decisions, so its latency is hidden too.  The decisions are
// band_segments', i.e. k_mc_band's and k_mc_quad's (same quad_cells on the
// same inputs).  Measured at 32 x 256^2 in FP32: 49 us per batched sweep
// against k_mc_quad's 30.7 -- 128 registers hold 2 CTAs (16 warps) per SM at
// 36-39 % issue, against k_mc_quad's 24 warps at 54 %, the top stall being
// the barrier that ends each item (ncu); taking the loads off the decisions'
// path does not pay where the decisions themselves are latency- and
// issue-bound and k_mc_quad's warps already hide its L2 loads.  Two segments
// per thread unrolled together: 51 us.  It is an autotuner candidate.
//
// Every wait on a buffer is bounded (MCP_WAIT_NS of the global timer): a warp
// whose wait runs out sets the CTA's abort flag and *err; after the item's
// barrier the CTA skips the remaining items, thread 0 waits (bounded again)
// for the copies still in flight, and the CTA returns; the host reads *err
// after the run.
constexpr int MCP_THREADS = 256;
constexpr int MCP_MIN_STAGES = 2;
constexpr int MCP_MAX_STAGES = 3;
constexpr int MCP_HDR = 128;  // bytes ahead of the stage buffers: the mbarriers, the abort flag
constexpr unsigned long long MCP_WAIT_NS = 2000000000ull;
__host__ __device__ inline bool mc_pipe_ok(const Geom& g) { return mc_band_ok(g); }
// rows per band: one 4-cell segment per thread (two, unrolled together so
// that their decisions interleave, measured no faster and spilled)
inline int mc_pipe_rows(const Geom& g) { return std::max(1, std::min(g.ny, 4 * MCP_THREADS / g.nx)); }
// elements of one stage buffer: m rows y0-1 .. y0+band, h rows y0 .. y0+band-1
__host__ __device__ inline size_t mc_pipe_stage_elems(const Geom& g, int band) {
  return (size_t)(2 * band + 2) * 3 * g.nx;
}
template <typename T>
inline size_t mc_pipe_smem(const Geom& g, int nst = MCP_MIN_STAGES) {
  return MCP_HDR + nst * mc_pipe_stage_elems(g, mc_pipe_rows(g)) * sizeof(T);
}

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ unsigned long long mcp_now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Waits until the phase with the given parity has completed, at most limit_ns.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = mcp_now_ns();
  while (!mbar_try_wait(bar, parity))
    if (mcp_now_ns() - t0 > limit_ns) return false;
  return true;
}
// Bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned) from
// global to shared memory, completing as transaction bytes on bar.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

// Warp 0: the copies of item i into buffer `buf` (see k_mc_pipe); dm: the
// item's replica has demag on (its h rows are needed).
template <typename T>
__device__ __forceinline__ void mc_pipe_issue(const Geom& g, const T* m, const T* h, int i, int band, int nbands,
                                              bool dm, T* buf, uint64_t* bar) {
  const int nx = g.nx, ny = g.ny;
  const long long n = g.n;
  const int r = i / nbands;
  const int y0 = (i - r * nbands) * band;
  const int nb = min(band, ny - y0);
  const bool wrap = g.per[1] && ny > 1;
  const int lo = (y0 > 0 || wrap) ? 0 : 1;             // first m slot present
  const int hi = (y0 + nb < ny || wrap) ? nb + 1 : nb;  // last m slot present
  const int nm = 3 * (hi - lo + 1), nh = dm ? 3 * nb : 0;
  const unsigned rowb = (unsigned)(nx * sizeof(T));
  const T* mr = m + (long long)r * 3 * n;
  const T* hr = h + (long long)r * 3 * n;
  T* hs = buf + (size_t)(band + 2) * 3 * nx;
  const int lane = threadIdx.x & 31;
  // the CTA's reads of this buffer (ordered before by a barrier) come before
  // the copies that overwrite it
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (lane == 0) mbar_arrive_expect_tx(bar, (unsigned)(nm + nh) * rowb);
  __syncwarp();
  for (int q = lane; q < nm + nh; q += 32) {
    if (q < nm) {
      const int slot = lo + q / 3, comp = q - (q / 3) * 3;
      int y = y0 - 1 + slot;
      if (y < 0) y += ny;
      else if (y >= ny) y -= ny;
      bulk_g2s(buf + ((size_t)slot * 3 + comp) * nx, mr + comp * n + (long long)y * nx, rowb, bar);
    } else {
      const int j = q - nm, rr = j / 3, comp = j - rr * 3;
      bulk_g2s(hs + ((size_t)rr * 3 + comp) * nx, hr + comp * n + (long long)(y0 + rr) * nx, rowb, bar);
    }
  }
}

__device__ __forceinline__ void flush_accepts(unsigned int& mine, unsigned long long* counter) {
  unsigned int v = mine;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(counter, (unsigned long long)v);
  mine = 0;
}

// m, h, acc and cp cover every replica (items = replicas x nbands); nst
// buffers (MCP_MIN_STAGES .. MCP_MAX_STAGES).
template <typename T, bool ALLB>
__global__ void __launch_bounds__(MCP_THREADS, 2)
    k_mc_pipe(Geom g, const McCoef<T>* __restrict__ cp, T* __restrict__ m, const T* __restrict__ h,
              const SweepCounters* __restrict__ ctr, int color, int band, int nbands, int items, int chunk, int nst,
              FastDiv dseg, unsigned long long* acc, int* err) {
  // no static shared memory: the dynamic limit is raised to the device's whole
  // opt-in size
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw);
  volatile int& abort_s = *reinterpret_cast<int*>(smem_raw + 64);
  T* buf0 = reinterpret_cast<T*>(smem_raw + MCP_HDR);
  const size_t selems = mc_pipe_stage_elems(g, band);
  const long long n = g.n;
  const int i0 = blockIdx.x * chunk, i1 = min(items, i0 + chunk);
  if (i0 >= i1) return;
  const bool producer = threadIdx.x < 32;
  if (threadIdx.x == 0) {
    for (int s = 0; s < nst; ++s) mbar_init(&bars[s], 1);
    abort_s = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  pdl_wait();  // m and h are the previous kernels' output
  if (producer)
    for (int k = 0; k < nst && i0 + k < i1; ++k)
      mc_pipe_issue<T>(g, m, h, i0 + k, band, nbands, cp[(i0 + k) / nbands].cd != (T)0, buf0 + k * selems,
                       &bars[k]);
  const uint32_t stage = ctr->stage, sweep = ctr->sweep;
  McCoef<T> c;
  int rc = -1;
  unsigned int mine = 0;
  int failed = -1;  // the item whose wait ran out
  for (int i = i0; i < i1; ++i) {
    const int k = i - i0, s = k % nst;
    const int inext = i + nst;
    const bool dm_next = producer && inext < i1 && cp[inext / nbands].cd != (T)0;
    // warp-uniform: every lane sees the phase complete, or the warp gives up
    const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(&bars[s], (unsigned)(k / nst) & 1u, MCP_WAIT_NS));
    if (!ok) {
      abort_s = 1;
    } else {
      const int r = i / nbands, y0 = (i - r * nbands) * band;
      if (r != rc) {
        if (rc >= 0) flush_accepts(mine, acc + rc);
        rc = r;
        c = cp[r];
      }
      const T* ms = buf0 + s * selems;
      band_segments<T, ALLB>(g, c, ms, ms + (size_t)(band + 2) * 3 * g.nx, m + (long long)r * 3 * n, y0,
                             min(band, g.ny - y0), color, c.cd != (T)0, dseg, stage, sweep, mine);
    }
    __syncthreads();  // buffer s is free; abort_s is final for this item
    if (abort_s) {
      failed = i;
      break;
    }
    if (producer && inext < i1) mc_pipe_issue<T>(g, m, h, inext, band, nbands, dm_next, buf0 + s * selems, &bars[s]);
  }
  if (rc >= 0) flush_accepts(mine, acc + rc);
  if (failed >= 0 && threadIdx.x == 0) {
    atomicExch(err, 1);
    // the copies still in flight: items failed .. failed + nst - 1
    for (int i = failed; i < min(i1, failed + nst); ++i) {
      const int k = i - i0;
      mbar_wait_bounded(&bars[k % nst], (unsigned)(k / nst) & 1u, MCP_WAIT_NS);
    }
  }
}

// Both colours of a two-colour film sweep (nz = 1) in one launch.  A CTA owns
// an MCT x MCT tile of one replica and holds, in shared memory, m on the tile
// plus a 2-cell margin and h on the tile plus a 1-cell margin.  Colour 0 runs
// on the tile and on the ring of cells next to it (without the corners): the
// ring cells belong to neighbouring tiles, and this CTA repeats, bit for bit,
// the decisions their owners make -- same inputs, same Philox counter -- so
// that colour 1 on the tile sees exactly the colour-0 state of the two-launch
// sweep.  Only tile cells are written back and counted.  Periodic axes must be
// whole tiles and at least two tiles long, so the margin never wraps onto the
// tile itself.
constexpr int MCT = 32;

// One 4- or 8-byte global -> shared copy through the async path (no register
// round trip, so a thread can have many in flight).
template <typename T>
__device__ __forceinline__ void cp_async_elem(T* smem, const T* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  if constexpr (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(gmem) : "memory");
}
constexpr int MCT_B = MCT + 4;  // m box side
constexpr int MCT_H = MCT + 2;  // h box side

__host__ __device__ inline bool mc_tile_ok(const Geom& g) {
  return g.nz == 1 && g.ncolors == 2 && (!g.per[0] || (g.nx % MCT == 0 && g.nx >= 2 * MCT)) &&
         (!g.per[1] || (g.ny % MCT == 0 && g.ny >= 2 * MCT));
}
template <typename T>
__host__ __device__ inline size_t mc_tile_smem() {
  return (size_t)3 * (MCT_B * MCT_B + MCT_H * MCT_H) * sizeof(T);
}

template <typename T>
__global__ void __launch_bounds__(256) k_mc_tile(Geom g, const McCoef<T>* __restrict__ cp, T* __restrict__ m,
                                                 const T* __restrict__ h, const SweepCounters* __restrict__ ctr,
                                                 unsigned long long* acc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);  // [comp][by][bx], MCT_B^2 per component
  T* sh = sm + 3 * MCT_B * MCT_B;           // [comp][hy][hx], MCT_H^2 per component
  __shared__ int colx[MCT_B], rowy[MCT_B];  // box column / row -> lattice x / y, -1 outside an open edge
  const McCoef<T> c = cp[blockIdx.z];
  const long long n = g.n;
  m += blockIdx.z * 3 * n;
  h += blockIdx.z * 3 * n;
  acc += blockIdx.z;
  const uint32_t stage = ctr->stage, sweep = ctr->sweep;
  const int x0 = blockIdx.x * MCT, y0 = blockIdx.y * MCT;
  if (threadIdx.x < MCT_B) {
    int v = x0 - 2 + (int)threadIdx.x;
    if (v < 0 || v >= g.nx) v = g.per[0] ? (v + g.nx) % g.nx : -1;
    colx[threadIdx.x] = v;
    int w = y0 - 2 + (int)threadIdx.x;
    if (w < 0 || w >= g.ny) w = g.per[1] ? (w + g.ny) % g.ny : -1;
    rowy[threadIdx.x] = w;
  }
  __syncthreads();
  constexpr int BB = MCT_B * MCT_B, HH = MCT_H * MCT_H;
  // asynchronous element copies, all in flight at once; cells outside an open
  // edge are zero
  for (int idx = threadIdx.x; idx < 3 * BB; idx += blockDim.x) {
    const int cc = idx / BB, r = idx - cc * BB, by = r / MCT_B, bx = r - by * MCT_B;
    const int gx = colx[bx], gy = rowy[by];
    if (gx >= 0 && gy >= 0)
      cp_async_elem<T>(sm + idx, m + cc * n + (long long)gy * g.nx + gx);
    else
      sm[idx] = (T)0;
  }
  const bool with_h = c.cd != (T)0;
  for (int idx = threadIdx.x; idx < 3 * HH; idx += blockDim.x) {
    const int cc = idx / HH, r = idx - cc * HH, hy = r / MCT_H, hx = r - hy * MCT_H;
    const int gx = colx[hx + 1], gy = rowy[hy + 1];
    if (with_h && gx >= 0 && gy >= 0)
      cp_async_elem<T>(sh + idx, h + cc * n + (long long)gy * g.nx + gx);
    else
      sh[idx] = (T)0;
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  __syncthreads();
  // one trial at box cell (bx, by); returns whether it was accepted
  auto trial = [&](int bx, int by) -> bool {
    const int gx = colx[bx], gy = rowy[by];
    if (gx < 0 || gy < 0) return false;
    Nbrs<T> nb;
    T* own = sm + by * MCT_B + bx;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int ex = bx + (s ? 1 : -1), ey = by + (s ? 1 : -1);
      const bool okx = colx[ex] >= 0, oky = rowy[ey] >= 0;
      nb.has[0][s] = okx;
      nb.has[1][s] = oky;
      nb.has[2][s] = false;
      const T* px = okx ? sm + by * MCT_B + ex : own;
      const T* py = oky ? sm + ey * MCT_B + bx : own;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        nb.v[0][s][k] = px[k * BB];
        nb.v[1][s][k] = py[k * BB];
        nb.v[2][s][k] = own[k * BB];
      }
    }
    const T* hp = sh + (by - 1) * MCT_H + (bx - 1);
    const Proposal<T> p = mc_propose<T>(c, (uint32_t)(gx + g.nx * gy), stage, sweep);
    if (mc_accept<T>(c, nb, own[0], own[BB], own[2 * BB], hp[0], hp[HH], hp[2 * HH], p)) {
      own[0] = p.x;
      own[BB] = p.y;
      own[2 * BB] = p.z;
      return true;
    }
    return false;
  };
  // the colour of box cell (bx, by) is (bx + by) & 1: x0 - 2 and y0 - 2 are even
  // and periodic axes have even length
  unsigned int mine = 0;
  // colour 0 on box rows 1 .. MCT + 2 (tile rows -1 .. MCT), box columns
  // 1 .. MCT + 2, without the four corners
  constexpr int HALF0 = (MCT + 2) / 2;
  for (int idx = threadIdx.x; idx < (MCT + 2) * HALF0; idx += blockDim.x) {
    const int by = 1 + idx / HALF0, k = idx - (by - 1) * HALF0;
    const int bx = 1 + 2 * k + ((by + 1) & 1);
    const bool edge_row = by == 1 || by == MCT + 2;
    if (edge_row && (bx == 1 || bx == MCT + 2)) continue;
    const bool acc_ok = trial(bx, by);
    if (acc_ok && by >= 2 && by < MCT + 2 && bx >= 2 && bx < MCT + 2) ++mine;
  }
  __syncthreads();
  // colour 1 on the tile
  constexpr int HALF1 = MCT / 2;
  for (int idx = threadIdx.x; idx < MCT * HALF1; idx += blockDim.x) {
    const int by = 2 + idx / HALF1, k = idx - (by - 2) * HALF1;
    const int bx = 2 + 2 * k + ((by + 1) & 1);
    if (trial(bx, by)) ++mine;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < 3 * MCT * MCT; idx += blockDim.x) {
    const int cc = idx / (MCT * MCT), r = idx - cc * MCT * MCT, ty = r / MCT, tx = r - ty * MCT;
    const int gx = colx[tx + 2], gy = rowy[ty + 2];
    if (gx >= 0 && gy >= 0 && x0 + tx < g.nx && y0 + ty < g.ny)
      m[cc * n + (long long)gy * g.nx + gx] = sm[cc * BB + (ty + 2) * MCT_B + tx + 2];
  }
  unsigned int v = mine;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(acc, (unsigned long long)v);
}

// Both colours of a two-colour film sweep (nz = 1, nx a multiple of 4) in one
// launch, by strips of rows.  A CTA owns `rows` consecutive rows of one
// replica (the last strip may be shorter) and stages the m rows y0 - 2 ..
// y0 + rows + 1 in shared memory (slot s holds row y0 - 2 + s, wrapped on a
// periodic y axis, absent beyond an open edge).  Colour 0 runs on its own
// rows and on the two rows next to them (y0 - 1 and y0 + rows): the owners of
// those rows make the same decisions from the same inputs, since the
// neighbours of a colour-0 cell are colour-1 cells, unchanged until colour 1.
// Colour 1 then runs on the own rows, reading the colour-0 values just
// decided.  A thread owns pairs of cells (2k, 2k + 1) of a row, one of each
// colour, and reads the pair's h once for both decisions.  The strip reads m
// from `m_in` and writes its own rows to `m_out`, a different buffer: other
// strips still read the rows it changes.  Each trial is mc_propose /
// mc_accept on the same inputs as in the per-colour forms, so the decisions
// are theirs bit for bit.  m is read once and written once per sweep, h is
// read once, and one launch replaces two.
constexpr int MCS_THREADS = 256;
constexpr int MCS_IPT = 4;  // own-row pairs per thread
__host__ __device__ inline bool mc_strip_ok(const Geom& g) {
  return g.nz == 1 && g.ncolors == 2 && g.nx % 4 == 0 && g.nx >= 4 && g.nx <= 2048;
}
// rows per strip: the own-row pairs of a strip fill the CTA's MCS_IPT pairs
// per thread, at most 32 rows
__host__ __device__ inline int mc_strip_rows(const Geom& g) {
  const int r = MCS_IPT * MCS_THREADS / (g.nx / 2);
  return r < 1 ? 1 : r > 32 ? 32 : (r > g.ny ? g.ny : r);
}
template <typename T>
__host__ __device__ inline size_t mc_strip_smem(const Geom& g) {
  return (size_t)(mc_strip_rows(g) + 4) * 3 * g.nx * sizeof(T);
}

// Lattice row of slot s of the strip starting at y0, or -1 (absent).
__device__ __forceinline__ int strip_slot_row(const Geom& g, int y0, int s) {
  int y = y0 - 2 + s;
  if (y < 0 || y >= g.ny) {
    if (!g.per[1]) return -1;
    y %= g.ny;
    if (y < 0) y += g.ny;
  }
  return y;
}

// One trial at x of slot s (lattice row y) with the given h; neighbours from
// the staged rows.  ALLB: every x and y bond exists.
template <typename T, bool ALLB>
__device__ __forceinline__ bool strip_trial(const Geom& g, const McCoef<T>& c, T* __restrict__ sm, int s, int y,
                                            int x, bool hdn, bool hup, T hx, T hy, T hz, uint32_t stage,
                                            uint32_t sweep) {
  const int nx = g.nx, rs = 3 * nx;
  T* own = sm + s * rs + x;
  int xl = x - 1, xr = x + 1;
  bool hl = true, hr = true;
  if (xl < 0) {
    if (g.per[0]) xl += nx;
    else hl = false;
  }
  if (xr >= nx) {
    if (g.per[0]) xr -= nx;
    else hr = false;
  }
  if constexpr (ALLB) hl = hr = hdn = hup = true;
  Nbrs<T> nb;
  nb.has[0][0] = hl;
  nb.has[0][1] = hr;
  nb.has[1][0] = hdn;
  nb.has[1][1] = hup;
  nb.has[2][0] = nb.has[2][1] = false;
  const T* row = sm + s * rs;
  T ov[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    ov[k] = own[k * nx];
    nb.v[0][0][k] = hl ? row[k * nx + xl] : ov[k];
    nb.v[0][1][k] = hr ? row[k * nx + xr] : ov[k];
    nb.v[1][0][k] = hdn ? own[k * nx - rs] : ov[k];
    nb.v[1][1][k] = hup ? own[k * nx + rs] : ov[k];
    nb.v[2][0][k] = nb.v[2][1][k] = ov[k];
  }
  const Proposal<T> p = mc_propose<T>(c, (uint32_t)(y * nx + x), stage, sweep);
  if (mc_accept<T>(c, nb, ov[0], ov[1], ov[2], hx, hy, hz, p)) {
    own[0] = p.x;
    own[nx] = p.y;
    own[2 * nx] = p.z;
    return true;
  }
  return false;
}

template <typename T>
struct Pair2 {
  T a, b;
};
template <typename T>
__device__ __forceinline__ Pair2<T> ld2(const T* p) {
  if constexpr (sizeof(T) == 4) {
    const float2 v = *reinterpret_cast<const float2*>(p);
    return {v.x, v.y};
  } else {
    const double2 v = *reinterpret_cast<const double2*>(p);
    return {v.x, v.y};
  }
}

template <typename T, bool ALLB>
__global__ void __launch_bounds__(MCS_THREADS) k_mc_strip(Geom g, const McCoef<T>* __restrict__ cp,
                                                          const T* __restrict__ m_in, T* __restrict__ m_out,
                                                          const T* __restrict__ h,
                                                          const SweepCounters* __restrict__ ctr, int rows,
                                                          FastDiv dq, FastDiv dp, unsigned long long* acc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);  // [slot][comp][x]
  pdl_wait();  // coefficients (tempering swaps), counters, m and h come from earlier kernels
  const McCoef<T> c = cp[blockIdx.z];
  const long long n = g.n;
  const int nx = g.nx, P = nx >> 1, Q = nx >> 2, rs = 3 * nx;
  const int y0 = blockIdx.x * rows;
  const int nown = min(rows, g.ny - y0);
  const int nslots = nown + 4;
  m_in += blockIdx.z * 3 * n;
  m_out += blockIdx.z * 3 * n;
  h += blockIdx.z * 3 * n;
  acc += blockIdx.z;
  const bool dm = c.cd != (T)0;
  const bool ybonds = g.ny > 1;
  const uint32_t stage = ctr->stage, sweep = ctr->sweep;
  // stage the slots (16-byte loads and stores, x fastest)
  for (int idx = threadIdx.x; idx < nslots * 3 * Q; idx += blockDim.x) {
    const int sk = dq.div(idx), q = idx - sk * Q;
    const int sl = sk / 3, k = sk - 3 * sl;
    const int y = strip_slot_row(g, y0, sl);
    if (y >= 0) st4<T>(sm + sl * rs + k * nx + 4 * q, ld4<T>(m_in + k * n + (long long)y * nx + 4 * q));
  }
  __syncthreads();
  // colour 0 on the own rows (slots 2 .. nown + 1), keeping the colour-1
  // cells' h for the second phase
  T h1[MCS_IPT][3];
  unsigned int mine = 0;
#pragma unroll
  for (int i = 0; i < MCS_IPT; ++i) {
    const int item = threadIdx.x + i * MCS_THREADS;
    if (item < nown * P) {
      const int r = dp.div(item), k = item - r * P;
      const int sl = 2 + r, y = y0 + r;
      const int p0 = y & 1;
      T hc[3] = {(T)0, (T)0, (T)0};
      if (dm) {
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) {
          const Pair2<T> hv = ld2<T>(h + cc * n + (long long)y * nx + 2 * k);
          hc[cc] = p0 ? hv.b : hv.a;
          h1[i][cc] = p0 ? hv.a : hv.b;
        }
      } else {
        h1[i][0] = h1[i][1] = h1[i][2] = (T)0;
      }
      const bool hdn = ybonds && (ALLB || strip_slot_row(g, y0, sl - 1) >= 0);
      const bool hup = ybonds && (ALLB || strip_slot_row(g, y0, sl + 1) >= 0);
      if (strip_trial<T, ALLB>(g, c, sm, sl, y, 2 * k + p0, hdn, hup, hc[0], hc[1], hc[2], stage, sweep)) ++mine;
    }
  }
  // colour 0 on the rows next to the strip (slots 1 and nown + 2): the
  // neighbouring strips' decisions, recomputed, not counted
  for (int item = threadIdx.x; item < 2 * P; item += blockDim.x) {
    const int side = item >= P, k = item - side * P;
    const int sl = side ? nown + 2 : 1;
    const int y = strip_slot_row(g, y0, sl);
    if (y < 0) continue;
    const int x = 2 * k + (y & 1);
    T hc[3] = {(T)0, (T)0, (T)0};
    if (dm) {
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) hc[cc] = h[cc * n + (long long)y * nx + x];
    }
    const bool hdn = ybonds && (ALLB || strip_slot_row(g, y0, sl - 1) >= 0);
    const bool hup = ybonds && (ALLB || strip_slot_row(g, y0, sl + 1) >= 0);
    strip_trial<T, ALLB>(g, c, sm, sl, y, x, hdn, hup, hc[0], hc[1], hc[2], stage, sweep);
  }
  __syncthreads();
  // colour 1 on the own rows
#pragma unroll
  for (int i = 0; i < MCS_IPT; ++i) {
    const int item = threadIdx.x + i * MCS_THREADS;
    if (item < nown * P) {
      const int r = dp.div(item), k = item - r * P;
      const int sl = 2 + r, y = y0 + r;
      const int p1 = (y & 1) ^ 1;
      const bool hdn = ybonds && (ALLB || strip_slot_row(g, y0, sl - 1) >= 0);
      const bool hup = ybonds && (ALLB || strip_slot_row(g, y0, sl + 1) >= 0);
      if (strip_trial<T, ALLB>(g, c, sm, sl, y, 2 * k + p1, hdn, hup, h1[i][0], h1[i][1], h1[i][2], stage, sweep))
        ++mine;
    }
  }
  __syncthreads();
  // own rows back, whole
  for (int idx = threadIdx.x; idx < nown * 3 * Q; idx += blockDim.x) {
    const int sk = dq.div(idx), q = idx - sk * Q;
    const int r = sk / 3, k = sk - 3 * r;
    st4<T>(m_out + k * n + (long long)(y0 + r) * nx + 4 * q, ld4<T>(sm + (r + 2) * rs + k * nx + 4 * q));
  }
  unsigned int v = mine;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(acc, (unsigned long long)v);
}

// =========================================================== energy
// Per-cell energies in FP64 whatever T is (calEnergyKernel,
// src/effective_H.h:35-43, + thrust::reduce, src/main.cu:945-948), reduced
// per block in a fixed order; a second single-block kernel sums the blocks.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Per-cell terms of the energy reduction: q[0..4] the five energies with the
// prefactors of e, q[5..7] m, q[8] (with_q) the solid angle of the two
// triangles of the plaquette at (x, y).
template <typename T>
__device__ __forceinline__ void energy_terms_at(const Geom& g, const EnCoef& e, const T* __restrict__ m,
                                                const T* __restrict__ h, long long i, bool with_q, double q[NQ]) {
  const long long n = g.n;
  const T* mx = m;
  const T* my = m + n;
  const T* mz = m + 2 * n;
  // cell coordinates by the multiply-shift dividers (n < 2^31)
  const int row = g.dnx.div((int)i), x = (int)i - row * g.nx;
  const int z = g.dny.div(row), y = row - z * g.ny;
  const double ax = mx[i], ay = my[i], az = mz[i];
  for (int a = 0; a < 3; ++a) {
    const long long j = nbr_idx(g, x, y, z, a, 1);
    if (j < 0) continue;
    const double ddx = (double)mx[j] - ax, ddy = (double)my[j] - ay, ddz = (double)mz[j] - az;
    q[0] += e.aexV_d2[a] * (ddx * ddx + ddy * ddy + ddz * ddz);
  }
  const long long xp = nbr_idx(g, x, y, z, 0, 1), xm = nbr_idx(g, x, y, z, 0, -1);
  const long long yp = nbr_idx(g, x, y, z, 1, 1), ym = nbr_idx(g, x, y, z, 1, -1);
  const double dxmz = (xp >= 0 ? (double)mz[xp] : 0.0) - (xm >= 0 ? (double)mz[xm] : 0.0);
  const double dxmx = (xp >= 0 ? (double)mx[xp] : 0.0) - (xm >= 0 ? (double)mx[xm] : 0.0);
  const double dymz = (yp >= 0 ? (double)mz[yp] : 0.0) - (ym >= 0 ? (double)mz[ym] : 0.0);
  const double dymy = (yp >= 0 ? (double)my[yp] : 0.0) - (ym >= 0 ? (double)my[ym] : 0.0);
  q[1] = -(ax * e.dV_2d[0] * dxmz + ay * e.dV_2d[1] * dymz - az * (e.dV_2d[0] * dxmx + e.dV_2d[1] * dymy));
  const double mu = ax * e.u[0] + ay * e.u[1] + az * e.u[2];
  q[2] = -e.kuV * mu * mu;
  q[3] = -(ax * e.msVB[0] + ay * e.msVB[1] + az * e.msVB[2]);
  if (e.demag != 0.0 && h) q[4] = -e.demag * (ax * (double)h[i] + ay * (double)h[n + i] + az * (double)h[2 * n + i]);
  q[5] = ax;
  q[6] = ay;
  q[7] = az;
  if (!with_q) return;
  const long long i2 = nbr_idx(g, x, y, z, 0, 1);
  const long long i4 = nbr_idx(g, x, y, z, 1, 1);
  if (i2 >= 0 && i4 >= 0) {
    const int x2 = (int)i2 - g.dnx.div((int)i2) * g.nx;
    const long long i3 = nbr_idx(g, x2, y, z, 1, 1);
    const long long tri[2][3] = {{i, i2, i3}, {i, i3, i4}};
    for (int t = 0; t < 2; ++t) {
      const long long a = tri[t][0], b = tri[t][1], cc = tri[t][2];
      const double pax = mx[a], pay = my[a], paz = mz[a];
      const double pbx = mx[b], pby = my[b], pbz = mz[b];
      const double pcx = mx[cc], pcy = my[cc], pcz = mz[cc];
      const double trip =
          pax * (pby * pcz - pbz * pcy) + pay * (pbz * pcx - pbx * pcz) + paz * (pbx * pcy - pby * pcx);
      const double den = 1.0 + (pax * pbx + pay * pby + paz * pbz) + (pbx * pcx + pby * pcy + pbz * pcz) +
                         (pcx * pax + pcy * pay + pcz * paz);
      q[8] += 2.0 * atan2(trip, den);
    }
  }
}

// Block sums of q[0..NQ) in a fixed order -> partials[blockIdx.x * NQ + k].
__device__ __forceinline__ void block_sum_nq(const double q[NQ], double* __restrict__ partials) {
  __shared__ double red[NQ][8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    const double v = warp_sum(q[k]);
    if (lane == 0) red[k][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x < NQ) {
    double s = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[threadIdx.x][w];
    partials[(long long)blockIdx.x * NQ + threadIdx.x] = s;
  }
}

// with_q = 0: the five energies (and m) only, without the solid angles of the
// topological charge -- FP64 atan2 per plaquette, the dearest part on a GPU
// whose FP64 rate is a small fraction of its FP32 rate; the energies are the
// same bit for bit.  Parallel-tempering swaps need only the energies.
template <typename T>
__global__ void __launch_bounds__(256) k_energy(Geom g, const EnCoef* __restrict__ ep, const T* __restrict__ m,
                                                const T* __restrict__ h, double* __restrict__ partials,
                                                int with_q) {
  const EnCoef e = ep[blockIdx.z];
  m += blockIdx.z * 3 * g.n;
  if (h) h += blockIdx.z * 3 * g.n;
  partials += (long long)blockIdx.z * gridDim.x * NQ;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double q[NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k) q[k] = 0;
  if (i < g.n) energy_terms_at<T>(g, e, m, h, i, with_q != 0, q);
  block_sum_nq(q, partials);
}

// The five energies of FP32 replicas for parallel-tempering swaps: each cell's
// terms in FP32 (the working precision of the replicas' own updates), summed
// per thread over ENL_CELLS cells in FP32 and from there in FP64.  Within
// ~1e-6 relative of the FP64-per-cell evaluation (k_energy) of the same state,
// far below what a swap decision resolves (kT ~ 1e-3 of these energies), at
// a small fraction of its cost on a GPU with a low FP64 rate.  q[5..8] are 0.
constexpr int ENL_CELLS = 8;
static __global__ void __launch_bounds__(256) k_energy_lean(Geom g, const EnCoef* __restrict__ ep,
                                                            const float* __restrict__ m, const float* __restrict__ h,
                                                            double* __restrict__ partials) {
  const EnCoef e = ep[blockIdx.z];
  const int n = (int)g.n;
  m += blockIdx.z * 3 * g.n;
  if (h) h += blockIdx.z * 3 * g.n;
  partials += (long long)blockIdx.z * gridDim.x * NQ;
  const float* mx = m;
  const float* my = m + n;
  const float* mz = m + 2 * n;
  const float aex[3] = {(float)e.aexV_d2[0], (float)e.aexV_d2[1], (float)e.aexV_d2[2]};
  const float dv0 = (float)e.dV_2d[0], dv1 = (float)e.dV_2d[1], kuv = (float)e.kuV;
  const float u0 = (float)e.u[0], u1 = (float)e.u[1], u2 = (float)e.u[2];
  const float b0 = (float)e.msVB[0], b1 = (float)e.msVB[1], b2 = (float)e.msVB[2];
  const float dmg = (float)e.demag;
  float acc[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int row = g.dnx.div(i), x = i - row * g.nx;
    const int z = g.dny.div(row), y = row - z * g.ny;
    const float ax = mx[i], ay = my[i], az = mz[i];
    for (int a = 0; a < 3; ++a) {
      const long long j = nbr_idx(g, x, y, z, a, 1);
      if (j < 0) continue;
      const float ddx = mx[j] - ax, ddy = my[j] - ay, ddz = mz[j] - az;
      acc[0] += aex[a] * (ddx * ddx + ddy * ddy + ddz * ddz);
    }
    const long long xp = nbr_idx(g, x, y, z, 0, 1), xm = nbr_idx(g, x, y, z, 0, -1);
    const long long yp = nbr_idx(g, x, y, z, 1, 1), ym = nbr_idx(g, x, y, z, 1, -1);
    const float dxmz = (xp >= 0 ? mz[xp] : 0.f) - (xm >= 0 ? mz[xm] : 0.f);
    const float dxmx = (xp >= 0 ? mx[xp] : 0.f) - (xm >= 0 ? mx[xm] : 0.f);
    const float dymz = (yp >= 0 ? mz[yp] : 0.f) - (ym >= 0 ? mz[ym] : 0.f);
    const float dymy = (yp >= 0 ? my[yp] : 0.f) - (ym >= 0 ? my[ym] : 0.f);
    acc[1] -= ax * dv0 * dxmz + ay * dv1 * dymz - az * (dv0 * dxmx + dv1 * dymy);
    const float mu = ax * u0 + ay * u1 + az * u2;
    acc[2] -= kuv * mu * mu;
    acc[3] -= ax * b0 + ay * b1 + az * b2;
    if (h) acc[4] -= dmg * (ax * h[i] + ay * h[n + i] + az * h[2 * n + i]);
  }
  double q[NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k) q[k] = k < 5 ? (double)acc[k] : 0.0;
  block_sum_nq(q, partials);
}

static __global__ void __launch_bounds__(256) k_reduce_partials(const double* __restrict__ partials, int nblocks,
                                                                double* __restrict__ out) {
  partials += (long long)blockIdx.x * nblocks * NQ;  // one block per replica
  out += blockIdx.x * NQ;
  __shared__ double red[NQ][8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = 0; k < NQ; ++k) {
    double s = 0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += partials[(long long)b * NQ + k];
    s = warp_sum(s);
    if (lane == 0) red[k][warp] = s;
  }
  __syncthreads();
  if (threadIdx.x < NQ) {
    double s = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[threadIdx.x][w];
    out[threadIdx.x] = s;
  }
}

// =========================================================== effective field
// Per-term H in A/m (the DEBUG_H_FIELD dumps of src/main.cu:965-1086).
// H of one term (0-4) or of all (5) at cell i, A/m.
template <typename T>
__device__ __forceinline__ void field_at(const Geom& g, const HCoef& c, int term, const T* __restrict__ m,
                                         const T* __restrict__ h, long long i, double f[3]) {
  const long long n = g.n;
  const T* mx = m;
  const T* my = m + n;
  const T* mz = m + 2 * n;
  // cell coordinates by the multiply-shift dividers (n < 2^31)
  const int row = g.dnx.div((int)i), x = (int)i - row * g.nx;
  const int z = g.dny.div(row), y = row - z * g.ny;
  const double ax = mx[i], ay = my[i], az = mz[i];
  double f0 = 0, f1 = 0, f2 = 0;
  const bool all = term == 5;
  if (term == 0 || all) {
    for (int a = 0; a < 3; ++a)
      for (int dir = -1; dir <= 1; dir += 2) {
        const long long j = nbr_idx(g, x, y, z, a, dir);
        if (j < 0) continue;
        f0 += c.ex_d2[a] * ((double)mx[j] - ax);
        f1 += c.ex_d2[a] * ((double)my[j] - ay);
        f2 += c.ex_d2[a] * ((double)mz[j] - az);
      }
  }
  if (term == 1 || all) {
    const long long xp = nbr_idx(g, x, y, z, 0, 1), xm = nbr_idx(g, x, y, z, 0, -1);
    const long long yp = nbr_idx(g, x, y, z, 1, 1), ym = nbr_idx(g, x, y, z, 1, -1);
    const double dxmz = (xp >= 0 ? (double)mz[xp] : 0.0) - (xm >= 0 ? (double)mz[xm] : 0.0);
    const double dxmx = (xp >= 0 ? (double)mx[xp] : 0.0) - (xm >= 0 ? (double)mx[xm] : 0.0);
    const double dymz = (yp >= 0 ? (double)mz[yp] : 0.0) - (ym >= 0 ? (double)mz[ym] : 0.0);
    const double dymy = (yp >= 0 ? (double)my[yp] : 0.0) - (ym >= 0 ? (double)my[ym] : 0.0);
    f0 += c.dm_2d[0] * dxmz;
    f1 += c.dm_2d[1] * dymz;
    f2 += -(c.dm_2d[0] * dxmx + c.dm_2d[1] * dymy);
  }
  if (term == 2 || all) {
    const double mu = ax * c.u[0] + ay * c.u[1] + az * c.u[2];
    f0 += c.an * mu * c.u[0];
    f1 += c.an * mu * c.u[1];
    f2 += c.an * mu * c.u[2];
  }
  if (term == 3 || all) {
    f0 += c.b[0];
    f1 += c.b[1];
    f2 += c.b[2];
  }
  if ((term == 4 || all) && c.ms != 0.0 && h) {
    f0 += c.ms * (double)h[i];
    f1 += c.ms * (double)h[n + i];
    f2 += c.ms * (double)h[2 * n + i];
  }
  f[0] = f0;
  f[1] = f1;
  f[2] = f2;
}

// Per-term H in A/m (the DEBUG_H_FIELD dumps of src/main.cu:965-1086).
template <typename T>
__global__ void k_field(Geom g, HCoef c, int term, const T* __restrict__ m, const T* __restrict__ h,
                        double* __restrict__ out) {
  const long long n = g.n;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double f[3];
  field_at<T>(g, c, term, m, h, i, f);
  out[i] = f[0];
  out[n + i] = f[1];
  out[2 * n + i] = f[2];
}

// =========================================================== init / utility
// Uniform directions from Philox(key = seed; counter = (i, 0, 0, STREAM_INIT)),
// computed in FP64 and rounded to T (replaces randInitMx, src/mx_init.h:21-97).
template <typename T>
__global__ void k_init(long long n, uint32_t k0, uint32_t k1, T* __restrict__ m) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  mmcm::u32x4 ctr = {(uint32_t)i, 0u, 0u, mmcm::STREAM_INIT};
  mmcm::u32x4 r = mmcm::philox4x32_10(ctr, k0, k1);
  double z = 2.0 * mmcm::u01_f64(r.x) - 1.0;
  double t = 1.0 - z * z;
  if (t < 0) t = 0;
  double s = mmcm::dsqrt(t), sn, cs;
  mmcm::sincospi(2.0 * mmcm::u01_f64(r.y), &sn, &cs);
  m[i] = (T)(s * cs);
  m[n + i] = (T)(s * sn);
  m[2 * n + i] = (T)z;
}

template <typename T>
__global__ void k_from_f64(long long n, const double* __restrict__ src, T* __restrict__ dst) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (T)src[i];
}
template <typename T>
__global__ void k_to_f64(long long n, const T* __restrict__ src, double* __restrict__ dst) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (double)src[i];
}
template <typename T>
__global__ void k_khat_store(long long count, const double2* __restrict__ src, C<T>* __restrict__ dst) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) dst[i] = cmk<C<T>>((T)src[i].x, (T)src[i].y);
}

// =========================================================== host launchers
#define MMC_TRY_ATTR(x)                  \
  do {                                   \
    cudaError_t e_ = (x);                \
    if (e_ != cudaSuccess) return e_;    \
  } while (0)
inline size_t x_pass_smem(const FftPlan& p, int lines_per_row, int rows, size_t csize) {
  return ((size_t)((p.tw_total + 1) & ~1) + 2 * (size_t)rows * lines_per_row * p.n) * csize;
}
inline size_t col_pass_smem_lean(const FftPlan& p, int ncomp, int tx, size_t csize) {
  return ((size_t)((p.tw_total + 1) & ~1) + (size_t)ncomp * tx * col_line_stride(p, csize)) * csize;
}
inline size_t col_pass_smem(const FftPlan& p, int ncomp, int tx, size_t csize, bool mul) {
  return ((size_t)((p.tw_total + 1) & ~1) + 2 * (size_t)ncomp * tx * col_line_stride(p, csize) +
          (mul ? 6 * (size_t)p.n * tx : 0)) *
         csize;
}
// Two line buffers and no tensor tile (the tensor read from global memory).
inline size_t col_pass_smem_kglobal(const FftPlan& p, int ncomp, int tx, size_t csize) {
  return col_pass_smem(p, ncomp, tx, csize, false);
}

// The warp-shaped x-pass kernels for the plan's (A, B), or null.
template <typename T>
struct XPassW {
  void (*fwd)(FftPlan, int, FastDiv, int, const T*, long long, C<T>*, long long, int, int, int, int, long long,
              long long);
  void (*inv)(FftPlan, const C<T>*, long long, int, int, int, FastDiv, FastDiv, int, T*, long long, int, long long,
              long long);
};
template <typename T>
XPassW<T> x_pass_w(const FftPlan& p) {
#define MMC_XW(A_, B_) \
  if (p.warp_a == A_ && p.warp_b == B_) return {k_x_forward_w<T, A_, B_>, k_x_inverse_w<T, A_, B_>};
  MMC_XW(32, 32)
  MMC_XW(32, 16)
  MMC_XW(16, 16)
  MMC_XW(16, 8)
  MMC_XW(8, 8)
  MMC_XW(16, 2)
  MMC_XW(8, 4)
#undef MMC_XW
  return {nullptr, nullptr};
}
inline size_t x_pass_w_smem(const FftPlan& p, int rows, size_t csize) {
  return ((size_t)p.n + 2 * (size_t)rows * (p.n + p.warp_a)) * csize;
}

// Raises the dynamic shared-memory limit of the FFT pass kernels to the
// device's opt-in maximum.  Called once per device at handle creation, never
// inside a stream capture.
template <typename T>
cudaError_t prepare_impl(int max_dyn_smem) {
  const void* fns[] = {(const void*)k_x_forward<T, false, 3>, (const void*)k_x_forward<T, true, 3>,
                       (const void*)k_x_forward<T, false, 6>, (const void*)k_x_forward<T, true, 6>,
                       (const void*)k_x_inverse<T, false>, (const void*)k_x_inverse<T, true>,
                       (const void*)k_col_pass<T, false>,      (const void*)k_col_pass<T, true>,
                       (const void*)k_col_pass_wide<T, false>, (const void*)k_col_pass_wide<T, true>};
  for (const void* f : fns) MMC_TRY_ATTR(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem));
  for (int s = 0; s < 7; ++s) {
    FftPlan p{};
    const int ab[7][2] = {{32, 32}, {32, 16}, {16, 16}, {16, 8}, {8, 8}, {16, 2}, {8, 4}};
    p.warp_a = ab[s][0];
    p.warp_b = ab[s][1];
    const XPassW<T> w = x_pass_w<T>(p);
    MMC_TRY_ATTR(cudaFuncSetAttribute((const void*)w.fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem));
    MMC_TRY_ATTR(cudaFuncSetAttribute((const void*)w.inv, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem));
  }
  MMC_TRY_ATTR(cudaFuncSetAttribute((const void*)k_mc_tile<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)mc_tile_smem<T>()));
  MMC_TRY_ATTR(cudaFuncSetAttribute((const void*)k_mc_band<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)MC_BAND_SMEM_MAX));
  MMC_TRY_ATTR(cudaFuncSetAttribute((const void*)k_mc_band<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)MC_BAND_SMEM_MAX));
  MMC_TRY_ATTR(cudaFuncSetAttribute((const void*)k_col_reg<T, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)col_reg_smem<T, 16>()));
  MMC_TRY_ATTR(cudaFuncSetAttribute((const void*)k_col_reg<T, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)col_reg_smem<T, 8>()));
  MMC_TRY_ATTR(cudaFuncSetAttribute((const void*)k_col_reg3<T, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)col_reg_smem<T, 16>()));
  MMC_TRY_ATTR(cudaFuncSetAttribute((const void*)k_col_reg3<T, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)col_reg_smem<T, 8>()));
  MMC_TRY_ATTR(cudaFuncSetAttribute((const void*)k_mc_strip<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    max_dyn_smem));
  MMC_TRY_ATTR(cudaFuncSetAttribute((const void*)k_mc_strip<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    max_dyn_smem));
  MMC_TRY_ATTR(cudaFuncSetAttribute((const void*)k_mc_pipe<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    max_dyn_smem));
  MMC_TRY_ATTR(cudaFuncSetAttribute((const void*)k_mc_pipe<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    max_dyn_smem));
  // the error word's address, looked up now rather than during a graph capture
  if (!mc_pipe_err_word()) return cudaErrorInvalidDevice;
  return cudaSuccess;
}

template <typename T>
cudaError_t run_x_forward(const FftPlan& p, int ncomp, int xdata, int ydata, int nrows, const T* in,
                          long long in_cstride, C<T>* S, long long nspec, int nyp, int hx, int pitch, int rpc,
                          int threads, cudaStream_t st, int nrep = 1, long long in_rstride = 0,
                          long long s_rstride = 0, bool inl = false) {
  if (ncomp == 3) {
    const XPassW<T> w = x_pass_w<T>(p);
    if (w.fwd) {
      dim3 grid((nrows + rpc - 1) / rpc, 1, nrep);
      return launch_pdl(w.fwd, grid, dim3(threads), x_pass_w_smem(p, rpc, sizeof(C<T>)), st, p, xdata,
                        FastDiv((uint32_t)ydata), nrows, in, in_cstride, S, nspec, nyp, hx, pitch, rpc, in_rstride,
                        s_rstride);
    }
  }
  if (ncomp == 3 && p.warp_a == 32) return cudaErrorInvalidValue;  // handled by k_x_forward_w above
  const int lines = (ncomp + 1) / 2;
  size_t sm = x_pass_smem(p, lines, rpc, sizeof(C<T>));
  dim3 grid((nrows + rpc - 1) / rpc, 1, nrep);
  if (ncomp != 3 && ncomp != 6) return cudaErrorInvalidValue;
  auto kern = ncomp == 3 ? (inl ? k_x_forward<T, true, 3> : k_x_forward<T, false, 3>)
                         : (inl ? k_x_forward<T, true, 6> : k_x_forward<T, false, 6>);
  kern<<<grid, threads, sm, st>>>(p, xdata, FastDiv((uint32_t)ydata), nrows, in, in_cstride, S, nspec, nyp,
                                  FastDiv((uint32_t)hx), pitch, rpc, in_rstride, s_rstride);
  return cudaGetLastError();
}

// The film column pass held in registers for a launch shape: 0 none, 1
// k_col_reg (col_lean 2), 2 k_col_reg3 (col_lean 3).
inline int col_regs(const DemagTuning& tun) { return tun.col_lean >= 2 ? tun.col_lean - 1 : 0; }
template <typename T>
cudaError_t run_col_pass(const FftPlan& p, int ncomp, C<T>* S, long long nspec, const C<T>* khat, int hx,
                         int planes, long long plane_stride, long long pos_stride, int load_lim, int store_lim,
                         int flags, T inv_n, int tx, int threads, cudaStream_t st, int nrep = 1,
                         long long s_rstride = 0, bool inl = false, bool lean = false, int regs = 0) {
  if (ncomp == 3 && p.n <= 16 && p.full_off > 0) {  // short lines: one thread per column
    const ColShortFn<T> ks = col_short_kernel<T>(p.n);
    if (ks) {
      dim3 grid((hx + 127) / 128, planes, nrep);
      return launch_pdl(ks, grid, dim3(128), 0, st, p, S, nspec, khat, hx, plane_stride, pos_stride, load_lim,
                        store_lim, flags, inv_n, s_rstride);
    }
  }
  if (regs && ncomp == 3 && planes == 1 && (flags & ~PASS_SYM) == (PASS_FWD | PASS_MUL | PASS_INV) &&
      pos_stride < (1LL << 31) && p.warp_a == p.warp_b && (p.warp_a == 16 || p.warp_a == 8)) {
    dim3 grid((hx + CR_TX - 1) / CR_TX, 1, nrep);
    if (regs == 2) {  // one component per thread
      if (p.warp_a == 16)
        return launch_pdl(k_col_reg3<T, 16>, grid, dim3(3 * CR_TX * 16), col_reg_smem<T, 16>(), st, p, S, nspec,
                          khat, hx, (int)pos_stride, load_lim, store_lim, flags, inv_n, s_rstride);
      return launch_pdl(k_col_reg3<T, 8>, grid, dim3(3 * CR_TX * 8), col_reg_smem<T, 8>(), st, p, S, nspec, khat,
                        hx, (int)pos_stride, load_lim, store_lim, flags, inv_n, s_rstride);
    }
    if (p.warp_a == 16)
      return launch_pdl(k_col_reg<T, 16>, grid, dim3(CR_TX * 16), col_reg_smem<T, 16>(), st, p, S, nspec, khat, hx,
                        (int)pos_stride, load_lim, store_lim, flags, inv_n, s_rstride);
    return launch_pdl(k_col_reg<T, 8>, grid, dim3(CR_TX * 8), col_reg_smem<T, 8>(), st, p, S, nspec, khat, hx,
                      (int)pos_stride, load_lim, store_lim, flags, inv_n, s_rstride);
  }
  if (tx < 1 || (tx & (tx - 1)) != 0 || threads % tx != 0) return cudaErrorInvalidValue;  // see k_col_pass
  // in-place transforms exist for the warp path only
  int lmode = lean && p.warp_a != 0 ? 1 : 0;
  size_t sm = lmode ? col_pass_smem_lean(p, ncomp, tx, sizeof(C<T>))
                    : col_pass_smem(p, ncomp, tx, sizeof(C<T>), (flags & PASS_MUL) != 0);
  if (!lmode && (flags & PASS_MUL) && sm > 48 * 1024) {
    // a tensor tile that does not fit beside the two line buffers is read from
    // global memory in the product instead (the same values, so the same results)
    int dev = 0, optin = 0;
    MMC_TRY_ATTR(cudaGetDevice(&dev));
    MMC_TRY_ATTR(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if (sm > (size_t)optin) {
      lmode = 2;
      sm = col_pass_smem_kglobal(p, ncomp, tx, sizeof(C<T>));
    }
  }
  dim3 grid((hx + tx - 1) / tx, planes, nrep);
  auto kern = p.warp_a == 32 ? (inl ? k_col_pass_wide<T, true> : k_col_pass_wide<T, false>)
                             : (inl ? k_col_pass<T, true> : k_col_pass<T, false>);
  // no more threads than the kernel's registers allow (the split of the work
  // does not change the results)
  cudaFuncAttributes fa;
  MMC_TRY_ATTR(cudaFuncGetAttributes(&fa, (const void*)kern));
  threads = std::min(threads, fa.maxThreadsPerBlock & ~31);
  threads -= threads % std::max(tx, 32);
  if (threads < 32) return cudaErrorInvalidValue;
  return launch_pdl(kern, grid, dim3(threads), sm, st, p, ncomp, S, nspec, khat, hx, plane_stride, pos_stride,
                    load_lim, store_lim, flags, inv_n, tx, s_rstride, lmode);
}

#define MMC_TRY(x)                       \
  do {                                   \
    cudaError_t e_ = (x);                \
    if (e_ != cudaSuccess) return e_;    \
  } while (0)

template <typename T>
cudaError_t demag_impl(const Geom& g, const FftPlan& px, const FftPlan& py, const FftPlan& pz,
                       const DemagTuning& tun, const T* m, T* h, void* spec, const void* khat, cudaStream_t st,
                       int nrep, cudaEvent_t* ev, int mul_flags = 0) {
  C<T>* S = reinterpret_cast<C<T>*>(spec);
  const C<T>* K = reinterpret_cast<const C<T>*>(khat);
  const long long ns = g.nspec;
  const long long mr = 3 * g.n, sr = 3 * ns;  // replica strides
  const T inv_n = (T)(1.0 / (double)g.np);
  const int rows = g.ny * g.nz;
  if (ev) MMC_TRY(cudaEventRecord(ev[0], st));
  MMC_TRY(run_x_forward<T>(px, 3, g.nx, g.ny, rows, m, g.n, S, ns, g.nyp, g.hx, g.hxp, tun.x_rows_per_cta,
                           tun.x_threads, st, nrep, mr, sr, tun.fft_inline != 0));
  if (ev) MMC_TRY(cudaEventRecord(ev[1], st));
  const long long ystride = g.hxp, yplane = (long long)g.nyp * g.hxp;
  if (g.nzp == 1) {
    MMC_TRY(run_col_pass<T>(py, 3, S, ns, K, g.hx, 1, yplane, ystride, g.ny, g.ny,
                            PASS_FWD | PASS_MUL | PASS_INV | mul_flags, inv_n, tun.col_tx, tun.col_threads, st, nrep,
                            sr, tun.fft_inline != 0, tun.col_lean != 0, col_regs(tun)));
  } else {
    MMC_TRY(run_col_pass<T>(py, 3, S, ns, K, g.hx, g.nz, yplane, ystride, g.ny, g.nyp, PASS_FWD, inv_n, tun.col_tx,
                            tun.col_threads, st, nrep, sr, tun.fft_inline != 0, tun.col_lean != 0));
    MMC_TRY(run_col_pass<T>(pz, 3, S, ns, K, g.hx, g.nyp, ystride, yplane, g.nz, g.nz,
                            PASS_FWD | PASS_MUL | PASS_INV | mul_flags, inv_n, tun.col_tx_z, tun.col_threads, st, nrep,
                            sr, tun.fft_inline != 0, tun.col_lean != 0));
    MMC_TRY(run_col_pass<T>(py, 3, S, ns, K, g.hx, g.nz, yplane, ystride, g.nyp, g.ny, PASS_INV, inv_n, tun.col_tx,
                            tun.col_threads, st, nrep, sr, tun.fft_inline != 0, tun.col_lean != 0));
  }
  if (ev) MMC_TRY(cudaEventRecord(ev[2], st));
  const int rpc = tun.x_rows_per_cta;
  dim3 grid((rows + rpc - 1) / rpc, 1, nrep);
  const XPassW<T> w = x_pass_w<T>(px);
  if (w.inv) {
    MMC_TRY(launch_pdl(w.inv, grid, dim3(tun.x_threads), x_pass_w_smem(px, rpc, sizeof(C<T>)), st, px,
                       (const C<T>*)S, ns, g.nyp, g.hx, g.hxp, g.dnx, g.dny, rows, h, g.n, rpc, sr, mr));
  } else {
    if (px.warp_a == 32) return cudaErrorInvalidValue;  // the wide shapes have warp-shaped x passes
    size_t sm = x_pass_smem(px, 2, rpc, sizeof(C<T>));
    auto kinv = tun.fft_inline ? k_x_inverse<T, true> : k_x_inverse<T, false>;
    kinv<<<grid, tun.x_threads, sm, st>>>(px, S, ns, g.nyp, g.hx, g.hxp, g.dnx, g.dny, rows, h, g.n, rpc, sr, mr);
  }
  MMC_TRY(cudaGetLastError());
  if (ev) MMC_TRY(cudaEventRecord(ev[3], st));
  return cudaSuccess;
}

template <typename T>
cudaError_t mc_impl(const Geom& g, const McCoef<T>* c, T* m, const T* h, const SweepCounters* ctr, int color,
                    unsigned long long* acc, cudaStream_t st, int nrep, int form) {
  const int threads = 256;
  // form: MC_FORM_TILE both colours in one tile launch, MC_FORM_QUAD one
  // vectorised launch per colour, else one scalar launch per colour
  if (color < 0) {  // every colour of the sweep
    if (form == MC_FORM_TILE && mc_tile_ok(g)) {
      dim3 grid((unsigned)((g.nx + MCT - 1) / MCT), (unsigned)((g.ny + MCT - 1) / MCT), nrep);
      k_mc_tile<T><<<grid, threads, mc_tile_smem<T>(), st>>>(g, c, m, h, ctr, acc);
      return cudaGetLastError();
    }
    for (int col = 0; col < g.ncolors; ++col) MMC_TRY(mc_impl<T>(g, c, m, h, ctr, col, acc, st, nrep, form));
    return cudaSuccess;
  }
  if (form == MC_FORM_PIPE && mc_pipe_ok(g)) {
    const int band = mc_pipe_rows(g);
    const int nbands = (g.ny + band - 1) / band;
    const long long items = (long long)nrep * nbands;
    auto kern = mc_all_bonds(g) ? k_mc_pipe<T, true> : k_mc_pipe<T, false>;
    int* err = mc_pipe_err_word();
    // the bulk copies need 16-byte aligned rows: nx * sizeof(T) is a multiple
    // of 16 (nx % 4 == 0), so aligned bases suffice
    if (!err || items > INT_MAX || ((uintptr_t)m | (uintptr_t)h) % 16 != 0) return cudaErrorInvalidValue;
    int dev = 0, nsm = 0, optin = 0, per_sm = 0;
    MMC_TRY(cudaGetDevice(&dev));
    MMC_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    MMC_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    // as many buffers as keep the CTAs per SM the registers allow (at most
    // MCP_MAX_STAGES, at least MCP_MIN_STAGES)
    int nst = MCP_MIN_STAGES;
    MMC_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, MCP_THREADS, mc_pipe_smem<T>(g, nst)));
    for (int k = nst + 1; k <= MCP_MAX_STAGES && mc_pipe_smem<T>(g, k) <= (size_t)optin; ++k) {
      int q = 0;
      MMC_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, kern, MCP_THREADS, mc_pipe_smem<T>(g, k)));
      if (q < per_sm) break;
      nst = k;
    }
    const size_t smem = mc_pipe_smem<T>(g, nst);
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    // a static chunk of consecutive items per CTA, every CTA resident at once
    const long long ctas = (long long)nsm * per_sm;
    const int chunk = (int)((items + ctas - 1) / ctas);
    const int grid = (int)((items + chunk - 1) / chunk);
    return launch_pdl(kern, dim3(grid), dim3(MCP_THREADS), smem, st, g, c, m, h, ctr, color, band, nbands,
                      (int)items, chunk, nst, FastDiv((uint32_t)(g.nx / 4)), acc, err);
  }
  if (form == MC_FORM_BAND && mc_band_ok(g)) {
    const int band = mc_band_rows<T>(g, threads);
    dim3 grid((unsigned)((g.ny + band - 1) / band), 1, nrep);
    auto kern = mc_all_bonds(g) ? k_mc_band<T, true> : k_mc_band<T, false>;
    kern<<<grid, threads, mc_band_smem<T>(g, band), st>>>(
        g, c, m, h, ctr, color, band, FastDiv((uint32_t)(g.nx * sizeof(T) / 16)), FastDiv((uint32_t)(g.nx / 4)), acc);
    return cudaGetLastError();
  }
  if (form == MC_FORM_QUAD && mc_quad_ok(g)) {
    // 128-thread CTAs: the same warps per SM as 256 (the registers limit
    // them), in finer pieces, measured 2 us faster per batched sweep
    const int qthreads = 128;
    const long long total = (long long)g.ny * g.nz * (g.nx >> 2);  // segments, two per thread
    dim3 grid((unsigned)((total + 2 * qthreads - 1) / (2 * qthreads)), 1, nrep);
    auto kern = g.nz > 1 ? (mc_all_bonds(g) ? k_mc_quad<T, true, true> : k_mc_quad<T, false, true>)
                         : (mc_all_bonds(g) ? k_mc_quad<T, true, false> : k_mc_quad<T, false, false>);
    return launch_pdl(kern, grid, dim3(qthreads), 0, st, g, c, m, h, ctr, color, acc);
  }
  if (g.ncolors == 2) {
    const long long total = (long long)g.ny * g.nz * ((g.nx + 1) / 2);
    dim3 grid((unsigned)((total + threads - 1) / threads), 1, nrep);
    MMC_TRY(launch_pdl(k_mc_checker<T>, grid, dim3(threads), 0, st, g, c, m, h, ctr, color, acc));
  } else {
    dim3 grid((unsigned)((g.n + threads - 1) / threads), 1, nrep);
    k_mc_general<T><<<grid, threads, 0, st>>>(g, c, m, h, ctr, color, acc);
  }
  return cudaGetLastError();
}

inline int energy_blocks(const Geom& g) { return (int)((g.n + 255) / 256); }

template <typename T>
cudaError_t energy_impl(const Geom& g, const EnCoef* e, const T* m, const T* h, double* partials, int npartials,
                        double* out, cudaStream_t st, int nrep, int with_q) {
  const int nb = energy_blocks(g);
  if (nb > npartials) return cudaErrorInvalidValue;
  k_energy<T><<<dim3(nb, 1, nrep), 256, 0, st>>>(g, e, m, h, partials, with_q);
  MMC_TRY(cudaGetLastError());
  k_reduce_partials<<<nrep, 256, 0, st>>>(partials, nb, out);
  return cudaGetLastError();
}

// with_q < 0: the energies for tempering swaps (k_energy_lean for FP32 replicas).
template <typename T>
cudaError_t energy_swap_impl(const Geom& g, const EnCoef* e, const T* m, const T* h, double* partials,
                             int npartials, double* out, cudaStream_t st, int nrep) {
  if constexpr (sizeof(T) == 4) {
    const int nb = std::max(1, energy_blocks(g) / ENL_CELLS);
    if (nb > npartials || g.n >= (1LL << 31)) return cudaErrorInvalidValue;
    k_energy_lean<<<dim3(nb, 1, nrep), 256, 0, st>>>(g, e, m, h, partials);
    MMC_TRY(cudaGetLastError());
    k_reduce_partials<<<nrep, 256, 0, st>>>(partials, nb, out);
    return cudaGetLastError();
  } else {
    return energy_impl<T>(g, e, m, h, partials, npartials, out, st, nrep, 0);
  }
}

template <typename T>
cudaError_t field_impl(const Geom& g, const HCoef& c, int term, const T* m, const T* h, double* out,
                       cudaStream_t st) {
  k_field<T><<<(unsigned)((g.n + 255) / 256), 256, 0, st>>>(g, c, term, m, h, out);
  return cudaGetLastError();
}

template <typename T>
cudaError_t init_impl(const Geom& g, uint64_t seed, T* m, cudaStream_t st) {
  k_init<T><<<(unsigned)((g.n + 255) / 256), 256, 0, st>>>(g.n, (uint32_t)(seed & 0xffffffffu),
                                                          (uint32_t)(seed >> 32), m);
  return cudaGetLastError();
}

// ----------------------------------------------------------- launcher bodies
// Explicitly instantiated for float in kernels_f32.cu and for double in kernels_f64.cu.
template <typename T>
cudaError_t launch_demag(const Geom& g, const FftPlan& px, const FftPlan& py, const FftPlan& pz,
                         const DemagTuning& tun, const T* m, T* h, void* spec, const void* khat, cudaStream_t st,
                         int nrep, cudaEvent_t* ev) {
  return demag_impl<T>(g, px, py, pz, tun, m, h, spec, khat, st, nrep, ev);
}
template <typename T>
cudaError_t launch_demag_sym(const Geom& g, const FftPlan& px, const FftPlan& py, const FftPlan& pz,
                             const DemagTuning& tun, const T* m, T* h, void* spec, const void* khat, cudaStream_t st) {
  return demag_impl<T>(g, px, py, pz, tun, m, h, spec, khat, st, 1, nullptr, PASS_SYM);
}
template <typename T>
cudaError_t launch_mc(const Geom& g, const McCoef<T>* c, T* m, const T* h, const SweepCounters* ctr, int color,
                      unsigned long long* acc, cudaStream_t st, int nrep, int form) {
  return mc_impl<T>(g, c, m, h, ctr, color, acc, st, nrep, form);
}
template <typename T>
cudaError_t launch_mc_strip(const Geom& g, const McCoef<T>* c, const T* m_in, T* m_out, const T* h,
                            const SweepCounters* ctr, unsigned long long* acc, cudaStream_t st, int nrep) {
  if (!mc_strip_ok(g) || m_in == m_out) return cudaErrorInvalidValue;
  const int rows = mc_strip_rows(g);
  dim3 grid((unsigned)((g.ny + rows - 1) / rows), 1, nrep);
  auto kern = mc_all_bonds(g) ? k_mc_strip<T, true> : k_mc_strip<T, false>;
  return launch_pdl(kern, grid, dim3(MCS_THREADS), mc_strip_smem<T>(g), st, g, c, m_in, m_out, h, ctr, rows,
                    FastDiv((uint32_t)(g.nx / 4)), FastDiv((uint32_t)(g.nx / 2)), acc);
}
template <typename T>
cudaError_t launch_energy(const Geom& g, const EnCoef* e, const T* m, const T* h, double* partials, int npartials,
                          double* out, cudaStream_t st, int nrep, int with_q) {
  if (with_q < 0) return energy_swap_impl<T>(g, e, m, h, partials, npartials, out, st, nrep);
  return energy_impl<T>(g, e, m, h, partials, npartials, out, st, nrep, with_q);
}
template <typename T>
cudaError_t launch_field(const Geom& g, const HCoef& c, int term, const T* m, const T* h, double* out,
                         cudaStream_t st) {
  return field_impl<T>(g, c, term, m, h, out, st);
}
template <typename T>
cudaError_t launch_init(const Geom& g, uint64_t seed, T* m, cudaStream_t st) {
  return init_impl<T>(g, seed, m, st);
}
template <typename T>
cudaError_t launch_col_pass_2d(const Geom& g, const FftPlan& py, const DemagTuning& tun, void* spec,
                               const void* khat, cudaStream_t st, int nrep) {
  const T inv_n = (T)(1.0 / (double)g.np);
  return run_col_pass<T>(py, 3, reinterpret_cast<C<T>*>(spec), g.nspec, reinterpret_cast<const C<T>*>(khat), g.hx, 1,
                         (long long)g.nyp * g.hxp, g.hxp, g.ny, g.ny, PASS_FWD | PASS_MUL | PASS_INV, inv_n,
                         tun.col_tx, tun.col_threads, st, nrep, 3 * g.nspec, tun.fft_inline != 0,
                         tun.col_lean != 0, col_regs(tun));
}
template <typename T>
cudaError_t launch_prepare(int max_dyn_smem) {
  return prepare_impl<T>(max_dyn_smem);
}
template <typename T>
cudaError_t launch_from_f64(long long count, const double* src, T* dst, cudaStream_t st) {
  if (count <= 0) return cudaSuccess;
  k_from_f64<T><<<(unsigned)((count + 255) / 256), 256, 0, st>>>(count, src, dst);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_to_f64(long long count, const T* src, double* dst, cudaStream_t st) {
  if (count <= 0) return cudaSuccess;
  k_to_f64<T><<<(unsigned)((count + 255) / 256), 256, 0, st>>>(count, src, dst);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_khat_store(long long count, const double2* spec64, void* khat, cudaStream_t st) {
  if (count <= 0) return cudaSuccess;
  k_khat_store<T><<<(unsigned)((count + 255) / 256), 256, 0, st>>>(count, spec64, reinterpret_cast<C<T>*>(khat));
  return cudaGetLastError();
}

#define MMC_INSTANTIATE_LAUNCHERS(T)                                                                          \
  template cudaError_t launch_demag<T>(const Geom&, const FftPlan&, const FftPlan&, const FftPlan&,           \
                                       const DemagTuning&, const T*, T*, void*, const void*, cudaStream_t, int, \
                                       cudaEvent_t*);                                                          \
  template cudaError_t launch_demag_sym<T>(const Geom&, const FftPlan&, const FftPlan&, const FftPlan&,       \
                                           const DemagTuning&, const T*, T*, void*, const void*, cudaStream_t); \
  template cudaError_t launch_mc<T>(const Geom&, const McCoef<T>*, T*, const T*, const SweepCounters*, int,   \
                                    unsigned long long*, cudaStream_t, int, int);                             \
  template cudaError_t launch_mc_strip<T>(const Geom&, const McCoef<T>*, const T*, T*, const T*,             \
                                          const SweepCounters*, unsigned long long*, cudaStream_t, int);       \
  template cudaError_t launch_energy<T>(const Geom&, const EnCoef*, const T*, const T*, double*, int, double*, \
                                        cudaStream_t, int, int);                                               \
  template cudaError_t launch_field<T>(const Geom&, const HCoef&, int, const T*, const T*, double*,            \
                                       cudaStream_t);                                                          \
  template cudaError_t launch_init<T>(const Geom&, uint64_t, T*, cudaStream_t);                               \
  template cudaError_t launch_prepare<T>(int);                                                                \
  template cudaError_t launch_col_pass_2d<T>(const Geom&, const FftPlan&, const DemagTuning&, void*, const void*, \
                                             cudaStream_t, int);                                              \
  template cudaError_t launch_from_f64<T>(long long, const double*, T*, cudaStream_t);                        \
  template cudaError_t launch_to_f64<T>(long long, const T*, double*, cudaStream_t);                          \
  template cudaError_t launch_khat_store<T>(long long, const double2*, void*, cudaStream_t);

}  // namespace mmc
