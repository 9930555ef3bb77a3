// grad.cuh -- adjoint of the total energy and projected-gradient relaxation.
//
// The energy (k_energy's five terms) is E(m) = -mu0 Ms V / 2 sum_i m_i . (A m)_i
// - Ms V sum_i m_i . B with A linear: exchange and DMI operators are symmetric
// (the central difference is antisymmetric, so the DMI block matrix is
// symmetric), anisotropy is local, and demag is the convolution with K.  The
// gradient with respect to the free components of m is therefore
//   dE/dm_i = -mu0 Ms V H_i,
// with H the effective field in which the demag part is the convolution with
// the symmetrised tensor (K(r) + K(-r)) / 2, whose spectrum is Re K^ (the
// adjoint of the demag convolution; PASS_SYM in the column pass).  No
// counterpart in the reference, which has no gradient.
//
// The scalar derivatives follow from the energy's form: exchange, DMI and
// anisotropy are linear in Aex, Dind and Ku1 (their derivatives are the
// energies at unit strength), Zeeman is linear and demag quadratic in Ms, and
// dE/dB = -Ms V sum m.
#pragma once
#include "kernels.cuh"

namespace mmc {

// grad (3n doubles, may be null) and per-block sums of
// [unit-Aex exchange, unit-Dind DMI, unit-Ku1 anisotropy, dE_zeeman/dMs,
//  dE_demag/dMs, sum mx, sum my, sum mz, 0] with eu holding the unit
// prefactors (V/d^2, V/(2d), V, V B, mu0 Ms V).
template <typename T>
__global__ void __launch_bounds__(256) k_grad(Geom g, HCoef c, EnCoef eu, double gscale, const T* __restrict__ m,
                                              const T* __restrict__ hs, double* __restrict__ grad,
                                              double* __restrict__ partials) {
  const long long n = g.n;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double q[NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k) q[k] = 0;
  if (i < n) {
    if (grad) {
      double f[3];
      field_at<T>(g, c, 5, m, hs, i, f);
      grad[i] = gscale * f[0];
      grad[n + i] = gscale * f[1];
      grad[2 * n + i] = gscale * f[2];
    }
    energy_terms_at<T>(g, eu, m, hs, i, false, q);
  }
  block_sum_nq(q, partials);
}

// ----------------------------------------------------------- relaxation
// Projected steepest descent with Barzilai-Borwein steps (Barzilai & Borwein,
// IMA J. Numer. Anal. 8, 1988; the projected form used for micromagnetic
// energy minimisation by Exl et al., J. Appl. Phys. 115, 2014).  With
// t = H / Ms the descent direction on the sphere is P = t - (t.m) m, and the
// torque |m x t| is the stopping measure.
constexpr int RELAX_NQ = 4;  // s.s, s.y, y.y, max |m x t|

// One evaluation.  P holds the previous direction on entry and this one on
// exit; s is the last update m_k - m_{k-1} (ignored when first != 0).
// y = g_k - g_{k-1} with g = -P.
template <typename T>
__global__ void __launch_bounds__(256) k_relax_eval(Geom g, HCoef c, double inv_ms, const T* __restrict__ m,
                                                    const T* __restrict__ hs, double* __restrict__ P,
                                                    const double* __restrict__ s, int first,
                                                    double* __restrict__ partials) {
  const long long n = g.n;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double ss = 0, sy = 0, yy = 0, tq = 0;
  if (i < n) {
    double f[3];
    field_at<T>(g, c, 5, m, hs, i, f);
    const double mx = m[i], my = m[n + i], mz = m[2 * n + i];
    const double tx = f[0] * inv_ms, ty = f[1] * inv_ms, tz = f[2] * inv_ms;
    const double cx = my * tz - mz * ty, cy = mz * tx - mx * tz, cz = mx * ty - my * tx;
    tq = sqrt(cx * cx + cy * cy + cz * cz);
    const double tm = tx * mx + ty * my + tz * mz;
    const double p[3] = {tx - tm * mx, ty - tm * my, tz - tm * mz};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (!first) {
        const double y = P[k * n + i] - p[k];  // (-p) - (-P_prev)
        const double sk = s[k * n + i];
        ss += sk * sk;
        sy += sk * y;
        yy += y * y;
      }
      P[k * n + i] = p[k];
    }
  }
  __shared__ double red[RELAX_NQ][8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double v[RELAX_NQ] = {ss, sy, yy, tq};
#pragma unroll
  for (int k = 0; k < RELAX_NQ; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double w = __shfl_down_sync(0xffffffffu, v[k], o);
      v[k] = k == 3 ? fmax(v[k], w) : v[k] + w;
    }
    if (lane == 0) red[k][warp] = v[k];
  }
  __syncthreads();
  if (threadIdx.x < RELAX_NQ) {
    double a = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
      a = threadIdx.x == 3 ? fmax(a, red[threadIdx.x][w]) : a + red[threadIdx.x][w];
    partials[(long long)blockIdx.x * RELAX_NQ + threadIdx.x] = a;
  }
}

static __global__ void __launch_bounds__(256) k_relax_reduce(const double* __restrict__ partials, int nblocks,
                                                             double* __restrict__ out) {
  __shared__ double red[RELAX_NQ][8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = 0; k < RELAX_NQ; ++k) {
    double a = 0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
      const double v = partials[(long long)b * RELAX_NQ + k];
      a = k == 3 ? fmax(a, v) : a + v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double w = __shfl_down_sync(0xffffffffu, a, o);
      a = k == 3 ? fmax(a, w) : a + w;
    }
    if (lane == 0) red[k][warp] = a;
  }
  __syncthreads();
  if (threadIdx.x < RELAX_NQ) {
    double a = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
      a = threadIdx.x == 3 ? fmax(a, red[threadIdx.x][w]) : a + red[threadIdx.x][w];
    out[threadIdx.x] = a;
  }
}

// m <- (m + tau P) / |m + tau P|; s <- new m - old m.
template <typename T>
__global__ void k_relax_update(long long n, T* __restrict__ m, const double* __restrict__ P, double tau,
                               double* __restrict__ s) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double mx = m[i], my = m[n + i], mz = m[2 * n + i];
  double ax = mx + tau * P[i], ay = my + tau * P[n + i], az = mz + tau * P[2 * n + i];
  const double r = 1.0 / sqrt(ax * ax + ay * ay + az * az);
  ax *= r;
  ay *= r;
  az *= r;
  const T nx = (T)ax, ny = (T)ay, nz = (T)az;
  s[i] = (double)nx - mx;
  s[n + i] = (double)ny - my;
  s[2 * n + i] = (double)nz - mz;
  m[i] = nx;
  m[n + i] = ny;
  m[2 * n + i] = nz;
}

// ----------------------------------------------------------- launchers
template <typename T>
cudaError_t launch_grad(const Geom& g, const HCoef& c, const EnCoef& eu, double gscale, const T* m, const T* hs,
                        double* grad, double* partials, int npartials, double* out, cudaStream_t st) {
  const int nb = (int)((g.n + 255) / 256);
  if (nb > npartials) return cudaErrorInvalidValue;
  k_grad<T><<<nb, 256, 0, st>>>(g, c, eu, gscale, m, hs, grad, partials);
  MMC_TRY(cudaGetLastError());
  k_reduce_partials<<<1, 256, 0, st>>>(partials, nb, out);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_relax_eval(const Geom& g, const HCoef& c, double inv_ms, const T* m, const T* hs, double* P,
                              const double* s, bool first, double* partials, int npartials, double* out,
                              cudaStream_t st) {
  const int nb = (int)((g.n + 255) / 256);
  if (nb * RELAX_NQ > npartials * NQ) return cudaErrorInvalidValue;
  k_relax_eval<T><<<nb, 256, 0, st>>>(g, c, inv_ms, m, hs, P, s, first ? 1 : 0, partials);
  MMC_TRY(cudaGetLastError());
  k_relax_reduce<<<1, 256, 0, st>>>(partials, nb, out);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_relax_update(const Geom& g, T* m, const double* P, double tau, double* s, cudaStream_t st) {
  k_relax_update<T><<<(unsigned)((g.n + 255) / 256), 256, 0, st>>>(g.n, m, P, tau, s);
  return cudaGetLastError();
}

#define MMC_INSTANTIATE_GRAD(T)                                                                                  \
  template cudaError_t launch_grad<T>(const Geom&, const HCoef&, const EnCoef&, double, const T*, const T*,      \
                                      double*, double*, int, double*, cudaStream_t);                            \
  template cudaError_t launch_relax_eval<T>(const Geom&, const HCoef&, double, const T*, const T*, double*,     \
                                            const double*, bool, double*, int, double*, cudaStream_t);          \
  template cudaError_t launch_relax_update<T>(const Geom&, T*, const double*, double, double*, cudaStream_t);

}  // namespace mmc
