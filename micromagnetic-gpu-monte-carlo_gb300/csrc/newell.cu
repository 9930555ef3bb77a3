// newell.cu -- FP64 Newell demag tensor with periodic images.
//
// The reference declares ktensorKernel2_step1 / _step2_div_const
// (src/demag_cu.h:20-28) without publishing their bodies; its complete CPU
// version is ktensorcpu::ktensorCPU (src/demag_cu.cu:119-248), which this
// kernel follows term for term: for each padded grid point the wrapped signed
// offset (:149-151), the image loops over [-max(pbc,0), max(pbc,0)] per axis
// (as the GPU orchestration src/main.cu:475-491 does), the 64 parity-signed
// evaluations of the f / g potentials of src/demag_cu.h:43-71 with the
// component argument permutations (:190-210), and the division by
// -4 pi dx dy dz (:221-228).  In the term form (tensor_sum = 0) one thread
// owns one grid point and accumulates in the reference's order; the node form
// (k_newell_nodes, the default) groups each image's terms by lattice node.  Elementary functions come from mmc_math.h and
// this file is compiled with -fmad=false, so the result is bit-identical to
// the CPU oracle's.
#include <cuda_runtime.h>

#include "mmc_internal.h"
#include "mmc_math.h"
#include "newell_far.h"

namespace mmc {

namespace {

__device__ __forceinline__ double absv(double x) { return x > 0 ? x : -x; }

__device__ __forceinline__ double newell_f(double x, double y, double z) {
  const double EPS = 1e-200;
  x = absv(x);
  y = absv(y);
  z = absv(z);
  const double R = mmcm::dsqrt(x * x + y * y + z * z);
  const double t1 = y / 2.0 * (z * z - x * x) * mmcm::asinh(y / (mmcm::dsqrt(x * x + z * z) + EPS));
  const double t2 = z / 2.0 * (y * y - x * x) * mmcm::asinh(z / (mmcm::dsqrt(x * x + y * y) + EPS));
  const double t3 = x * y * z * mmcm::atan(y * z / (x * R + EPS));
  const double t4 = 1.0 / 6.0 * (2 * x * x - y * y - z * z) * R;
  return t1 + t2 - t3 + t4;
}

__device__ __forceinline__ double newell_g(double x, double y, double z) {
  const double EPS = 1e-200;
  z = absv(z);
  const double R = mmcm::dsqrt(x * x + y * y + z * z);
  const double t1 = x * y * z * mmcm::asinh(z / (mmcm::dsqrt(x * x + y * y) + EPS));
  const double t2 = y / 6.0 * (3.0 * z * z - y * y) * mmcm::asinh(x / (mmcm::dsqrt(y * y + z * z) + EPS));
  const double t3 = x / 6.0 * (3.0 * z * z - x * x) * mmcm::asinh(y / (mmcm::dsqrt(x * x + z * z) + EPS));
  const double t4 = z * z * z / 6.0 * mmcm::atan(x * y / (z * R + EPS));
  const double t5 = z * y * y / 2.0 * mmcm::atan(x * z / (y * R + EPS));
  const double t6 = z * x * x / 2.0 * mmcm::atan(y * z / (x * R + EPS));
  const double t7 = x * y * R / 3.0;
  return t1 + t2 + t3 - t4 - t5 - t6 - t7;
}

__device__ __forceinline__ int wrap_offset(int x, int n) { return (x + (n + 1) / 2 - 1) % n - (n + 1) / 2 + 1; }

// Adds images px in [px0, px1] (all py, pz) to the running sums of every
// point.  The sums live in k6 between launches, so splitting the image range
// over several launches keeps the reference's summation order exactly; the
// launch with `finalize` divides by -4 pi dx dy dz.
// far_r2 > 0: image offsets with |r|^2 >= far_r2 use the far-field expansion
// (newell_far.h) in place of the 64 terms.
__global__ void __launch_bounds__(128) k_newell(int nxp, int nyp, int nzp, double dx, double dy, double dz, int Px,
                                                int Py, int Pz, int px0, int px1, int finalize, double pi,
                                                double far_r2, double* __restrict__ k6, long long np) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const int x = (int)(i % nxp), y = (int)((i / nxp) % nyp), z = (int)(i / ((long long)nxp * nyp));
  const int idx_x = wrap_offset(x, nxp), idx_y = wrap_offset(y, nyp), idx_z = wrap_offset(z, nzp);
  double kxx = 0, kxy = 0, kxz = 0, kyy = 0, kyz = 0, kzz = 0;
  if (px0 > -Px) {
    kxx = k6[i];
    kxy = k6[np + i];
    kxz = k6[2 * np + i];
    kyy = k6[3 * np + i];
    kyz = k6[4 * np + i];
    kzz = k6[5 * np + i];
  }
  for (int px = px0; px <= px1; px++)
    for (int py = -Py; py <= Py; py++)
      for (int pz = -Pz; pz <= Pz; pz++) {
        const int ix = idx_x + px * nxp, iy = idx_y + py * nyp, iz = idx_z + pz * nzp;
        if (far_r2 > 0.0) {
          const double X = ix * dx, Y = iy * dy, Z = iz * dz;
          if (X * X + Y * Y + Z * Z >= far_r2) {
            double r[6];
            mmcm::newell_far_raw(X, Y, Z, dx, dy, dz, r);
            kxx += r[0];
            kxy += r[1];
            kxz += r[2];
            kyy += r[3];
            kyz += r[4];
            kzz += r[5];
            continue;
          }
        }
#pragma unroll 1
        for (int bits = 0; bits < 64; ++bits) {
          // bit order matches the nested FOR01 loops ikx, iky, ikz, ilx, ily, ilz
          const int ikx = (bits >> 5) & 1, iky = (bits >> 4) & 1, ikz = (bits >> 3) & 1;
          const int ilx = (bits >> 2) & 1, ily = (bits >> 1) & 1, ilz = bits & 1;
          const int iix = ix + ikx - ilx, iiy = iy + iky - ily, iiz = iz + ikz - ilz;
          const bool sign = ((ikx + iky + ikz + ilx + ily + ilz) % 2 == 0);
          const double X = iix * dx, Y = iiy * dy, Z = iiz * dz;
          double v;
          v = newell_f(X, Y, Z);
          kxx += sign ? v : -v;
          v = newell_g(X, Y, Z);
          kxy += sign ? v : -v;
          v = newell_g(X, Z, Y);
          kxz += sign ? v : -v;
          v = newell_f(Y, Z, X);
          kyy += sign ? v : -v;
          v = newell_g(Y, Z, X);
          kyz += sign ? v : -v;
          v = newell_f(Z, X, Y);
          kzz += sign ? v : -v;
        }
      }
  if (finalize) {
    const double d = -pi * 4.0 * dx * dy * dz;
    kxx = kxx / d;
    kxy = kxy / d;
    kxz = kxz / d;
    kyy = kyy / d;
    kyz = kyz / d;
    kzz = kzz / d;
  }
  k6[i] = kxx;
  k6[np + i] = kxy;
  k6[2 * np + i] = kxz;
  k6[3 * np + i] = kyy;
  k6[4 * np + i] = kyz;
  k6[5 * np + i] = kzz;
}

// The node form (tensor_sum = 1).  Per axis the parity-signed terms over
// (ik, il) in {0,1}^2 of the 64-term sum are the weights 2 at s = ik - il = 0
// and -1 at s = +-1, so one image's sum at offset o is
//   sum over s in {-1,0,1}^3 of w(sx) w(sy) w(sz) F(o + s)
// (sx outer, sz inner; each w F exact), and the six potentials F at a
// lattice node serve the 27 offsets around it.  A CTA owns a tile of
// NT x NT offsets (x, y) at one z offset; per image it evaluates the six
// potentials on the tile's nodes and one node around it (3 z layers) into
// shared memory -- 972 nodes against 256 x 64 terms -- and each thread forms
// its offset's 27-term sum from there and adds it to its running sum.  Image
// offsets at least the far radius away use the far-field expansion, and a
// tile whose every offset is that far skips its nodes.  The oracle's
// newell_point_nodes is the same arithmetic in the same order.
constexpr int NT = 16;
__device__ __forceinline__ double box_min_sq(int lo, int hi, double d) {
  if (lo <= 0 && hi >= 0) return 0.0;
  const double v = (lo > 0 ? lo : -hi) * d;
  return v * v;
}

__global__ void __launch_bounds__(NT * NT) k_newell_nodes(int nxp, int nyp, int nzp, double dx, double dy,
                                                          double dz, int Px, int Py, int Pz, int px0, int px1,
                                                          int finalize, double pi, double far_r2,
                                                          double* __restrict__ k6, long long np) {
  constexpr int NW = NT + 2;
  __shared__ double F[6][3][NW][NW];
  const int tx = threadIdx.x % NT, ty = threadIdx.x / NT;
  const int omx = 1 - (nxp + 1) / 2, omy = 1 - (nyp + 1) / 2, omz = 1 - (nzp + 1) / 2;  // smallest offsets
  const int bx = omx + blockIdx.x * NT, by = omy + blockIdx.y * NT;                    // the tile's first
  const int ox = bx + tx, oy = by + ty, oz = omz + (int)blockIdx.z;
  const bool inside = ox - omx < nxp && oy - omy < nyp;
  const long long i = inside ? (long long)((ox + nxp) % nxp) +
                                   (long long)nxp * ((oy + nyp) % nyp + (long long)nyp * ((oz + nzp) % nzp))
                             : 0;
  double k[6] = {0, 0, 0, 0, 0, 0};
  if (inside && px0 > -Px)
    for (int c = 0; c < 6; ++c) k[c] = k6[c * np + i];
  const double w1[3] = {-1.0, 2.0, -1.0};
  for (int px = px0; px <= px1; px++)
    for (int py = -Py; py <= Py; py++)
      for (int pz = -Pz; pz <= Pz; pz++) {
        const int ix = ox + px * nxp, iy = oy + py * nyp, iz = oz + pz * nzp;
        const int ex = bx + px * nxp, ey = by + py * nyp;  // the tile's first offsets of this image
        const bool tile_far = far_r2 > 0.0 && box_min_sq(ex, ex + NT - 1, dx) + box_min_sq(ey, ey + NT - 1, dy) +
                                                      box_min_sq(iz, iz, dz) >= far_r2;
        if (!tile_far) {
          __syncthreads();  // the previous image's stencils have read F
          for (int n = threadIdx.x; n < 3 * NW * NW; n += blockDim.x) {
            const int lz = n / (NW * NW), r = n - lz * NW * NW, ly = r / NW, lx = r - ly * NW;
            const double X = (ex - 1 + lx) * dx, Y = (ey - 1 + ly) * dy, Z = (iz - 1 + lz) * dz;
            F[0][lz][ly][lx] = newell_f(X, Y, Z);
            F[1][lz][ly][lx] = newell_g(X, Y, Z);
            F[2][lz][ly][lx] = newell_g(X, Z, Y);
            F[3][lz][ly][lx] = newell_f(Y, Z, X);
            F[4][lz][ly][lx] = newell_g(Y, Z, X);
            F[5][lz][ly][lx] = newell_f(Z, X, Y);
          }
          __syncthreads();
        }
        if (!inside) continue;
        if (far_r2 > 0.0) {
          const double X = ix * dx, Y = iy * dy, Z = iz * dz;
          if (X * X + Y * Y + Z * Z >= far_r2) {
            double r[6];
            mmcm::newell_far_raw(X, Y, Z, dx, dy, dz, r);
            for (int c = 0; c < 6; ++c) k[c] += r[c];
            continue;
          }
        }
        double a[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int sx = -1; sx <= 1; ++sx)
#pragma unroll
          for (int sy = -1; sy <= 1; ++sy)
#pragma unroll
            for (int sz = -1; sz <= 1; ++sz) {
              const double w = w1[sx + 1] * w1[sy + 1] * w1[sz + 1];
#pragma unroll
              for (int c = 0; c < 6; ++c) a[c] += w * F[c][1 + sz][1 + ty + sy][1 + tx + sx];
            }
        for (int c = 0; c < 6; ++c) k[c] += a[c];
      }
  if (!inside) return;
  if (finalize) {
    const double d = -pi * 4.0 * dx * dy * dz;
    for (int c = 0; c < 6; ++c) k[c] = k[c] / d;
  }
  for (int c = 0; c < 6; ++c) k6[c * np + i] = k[c];
}

}  // namespace

cudaError_t launch_newell(const Geom& g, double dx, double dy, double dz, int Px, int Py, int Pz, double pi,
                          double* k6, int px0, int px1, int finalize, cudaStream_t st, double far_r2, int nodes) {
  if (nodes && g.tzp <= 65535 && (g.typ + NT - 1) / NT <= 65535) {  // grid y and z limits; else the term form
    dim3 grid((unsigned)((g.txp + NT - 1) / NT), (unsigned)((g.typ + NT - 1) / NT), (unsigned)g.tzp);
    k_newell_nodes<<<grid, NT * NT, 0, st>>>(g.txp, g.typ, g.tzp, dx, dy, dz, Px, Py, Pz, px0, px1, finalize, pi,
                                             far_r2, k6, g.tnp);
    return cudaGetLastError();
  }
  const int threads = 128;
  k_newell<<<(unsigned)((g.tnp + threads - 1) / threads), threads, 0, st>>>(
      g.txp, g.typ, g.tzp, dx, dy, dz, Px, Py, Pz, px0, px1, finalize, pi, far_r2, k6, g.tnp);
  return cudaGetLastError();
}

namespace {
// Index on the tensor grid (extent t) of transform-grid index j (extent f) of
// an axis with n cells, or -1 where the transform grid holds no offset of the
// tensor.
__device__ __forceinline__ int rewrap_index(int j, int f, int t, int n) {
  if (f == t || j <= n - 1) return j;
  if (j >= f - (n - 1)) return j - f + t;
  return -1;
}

__global__ void k_tensor_rewrap(const double* __restrict__ k6t, long long tnp, int tx, int ty, int tz, int nx,
                                int ny, int nz, double* __restrict__ k6f, int fx, int fy, int fz, long long fnp) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= fnp) return;
  const int jx = (int)(i % fx), jy = (int)((i / fx) % fy), jz = (int)(i / ((long long)fx * fy));
  const int ix = rewrap_index(jx, fx, tx, nx), iy = rewrap_index(jy, fy, ty, ny), iz = rewrap_index(jz, fz, tz, nz);
  const bool ok = ix >= 0 && iy >= 0 && iz >= 0;
  const long long src = ok ? ix + (long long)tx * (iy + (long long)ty * iz) : 0;
  for (int c = 0; c < 6; ++c) k6f[c * fnp + i] = ok ? k6t[c * tnp + src] : 0.0;
}
}  // namespace

cudaError_t launch_tensor_rewrap(const Geom& g, const double* k6t, double* k6f, cudaStream_t st) {
  const int threads = 256;
  k_tensor_rewrap<<<(unsigned)((g.np + threads - 1) / threads), threads, 0, st>>>(
      k6t, g.tnp, g.txp, g.typ, g.tzp, g.nx, g.ny, g.nz, k6f, g.nxp, g.nyp, g.nzp, g.np);
  return cudaGetLastError();
}

}  // namespace mmc
