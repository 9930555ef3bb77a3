// oracle.cpp -- FP64 CPU restatement of the micromagnetic Monte Carlo hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle used by
// tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  The
// product (libmmc) never links, loads or calls it.
//
// Parity status: pinned to the reference's own code where the reference has
// any.  Its complete demag arithmetic -- ktensorCPU, f, g and
// calHexchangeKernel (src/demag_cu.cu, src/demag_cu.h) -- compiles unmodified
// with stand-in headers (oracle/build_ref.py -> oracle/_ref); its outputs are
// committed in tests/golden/ref_demag_golden.npz, and this file built with
// -DORACLE_LIBM (C library functions, its own Philox) reproduces the tensor
// and the product bit for bit (tests/test_ref_pin.py).  The reference's
// Metropolis, energy and self-tensor kernels have no published bodies; for
// those this file follows the physics contract below and is pinned by the
// Random123 known-answer vectors for Philox4x32-10, high-precision (mpmath)
// evaluations of the Newell formulas (tests/golden/) and physics identities
// (self-tensor trace, local dE == global energy difference, FFT convolution
// == direct sum).
//
// What follows the reference line by line:
//  - newell_f / newell_g: src/demag_cu.h:43-71 (same expression order).
//  - newell_tensor: ktensorCPU, src/demag_cu.cu:119-248 -- offset wrap
//    (:149-151), image loops over [-max(pbc,0), max(pbc,0)] as the GPU
//    orchestration src/main.cu:475-491 does, the 64-term parity-signed sum
//    (:170-213) and the division by -4*pi*dx*dy*dz (:221-228); with
//    tensor_sum = 1 each image's 64 terms grouped by lattice node
//    (newell_point_nodes), the library's default form.
//  - demag product: calHexchangeKernel, src/demag_cu.cu:68-116 (K^ . M^ / N).
//  - padding: src/main.cu:254-263.
// What follows the physics contract this project fixes for the missing
// kernels (mcKernel2, calEnergyKernel, calDemagMirrorTensor): exchange, DMI,
// anisotropy, Zeeman and demag energies, the sublattice Metropolis sweep and
// the Philox-keyed proposals.  Elementary functions come from mmc_math.h so
// that FP64 results can be compared bit for bit; compile with
// -ffp-contract=off.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/mmc.h"

#ifdef ORACLE_LIBM
// Independent build (liboracle_libm.so): the C library's elementary functions
// and a Philox4x32-10 written here from Salmon, Moraes, Dror, Shaw, "Parallel
// random numbers: as easy as 1, 2, 3" (SC'11), so that nothing of the
// product's csrc/mmc_math.h enters.  Its tensor equals the reference's own
// ktensorCPU bit for bit (same libm, same expression and loop order); the
// default build is checked against it to the rounding of one ulp per
// elementary function.  The far-field tensor form is not offered here.
namespace om {
inline double dsqrt(double x) { return std::sqrt(x); }
inline double asinh(double x) { return std::asinh(x); }
inline double atan(double x) { return std::atan(x); }
inline double exp(double x) { return std::exp(x); }
inline double log(double x) { return std::log(x); }
inline void sincospi(double t, double* s, double* c) {
  const double a = 3.14159265358979323846 * t;
  *s = std::sin(a);
  *c = std::cos(a);
}
struct u32x4 {
  uint32_t x, y, z, w;
};
// Counter word 3 of the keying contract: sweeps use 0, the initial state 1.
enum : uint32_t { STREAM_SWEEP = 0u, STREAM_INIT = 1u };
inline u32x4 philox4x32_10(u32x4 c, uint32_t k0, uint32_t k1) {
  for (int round = 0; round < 10; ++round) {
    if (round > 0) {
      k0 += 0x9E3779B9u;  // Weyl increments of the key
      k1 += 0xBB67AE85u;
    }
    const uint64_t a = (uint64_t)0xD2511F53u * (uint64_t)c.x;
    const uint64_t b = (uint64_t)0xCD9E8D57u * (uint64_t)c.z;
    u32x4 n;
    n.x = (uint32_t)(b >> 32) ^ c.y ^ k0;
    n.y = (uint32_t)b;
    n.z = (uint32_t)(a >> 32) ^ c.w ^ k1;
    n.w = (uint32_t)a;
    c = n;
  }
  return c;
}
inline double u01_f64(uint32_t r) { return ((double)r + 0.5) * 0x1p-32; }
}  // namespace om
#else
#include "../micromagnetic-gpu-monte-carlo_gb300/csrc/mmc_math.h"
#include "../micromagnetic-gpu-monte-carlo_gb300/csrc/newell_far.h"
namespace om = mmcm;
#endif

namespace {

const double kB = 1.3806488e-23;  // src/constant.h:22

double pi_of(const mmc_config* c) { return c->use_reference_pi ? 3.14159265358 : 3.14159265358979323846; }

struct Lat {
  int nx, ny, nz;
  int nxp, nyp, nzp;
  bool per[3];
  int P[3];
  long n() const { return (long)nx * ny * nz; }
  long np() const { return (long)nxp * nyp * nzp; }
};

Lat lat_of(const mmc_config* c) {
  Lat L;
  L.nx = c->nx; L.ny = c->ny; L.nz = c->nz;
  // src/main.cu:254-260: open axes (pbc == 0) are padded to 2n-1.
  L.nxp = c->pbc_x == 0 ? 2 * c->nx - 1 : c->nx;
  L.nyp = c->pbc_y == 0 ? 2 * c->ny - 1 : c->ny;
  L.nzp = c->pbc_z == 0 ? 2 * c->nz - 1 : c->nz;
  L.per[0] = c->pbc_x != 0; L.per[1] = c->pbc_y != 0; L.per[2] = c->pbc_z != 0;
  L.P[0] = c->pbc_x > 0 ? c->pbc_x : 0;
  L.P[1] = c->pbc_y > 0 ? c->pbc_y : 0;
  L.P[2] = c->pbc_z > 0 ? c->pbc_z : 0;
  return L;
}

// ---------------------------------------------------------------- Newell
double ABSV(double x) { return x > 0 ? x : -x; }  // src/constant.h:17

// src/demag_cu.h:43-56
double newell_f(double x, double y, double z) {
  const double EPS = 1e-200;  // src/constant.h:23
  x = ABSV(x);
  y = ABSV(y);
  z = ABSV(z);
  double R = om::dsqrt(x * x + y * y + z * z);
  double t1 = y / 2.0 * (z * z - x * x) * om::asinh(y / (om::dsqrt(x * x + z * z) + EPS));
  double t2 = z / 2.0 * (y * y - x * x) * om::asinh(z / (om::dsqrt(x * x + y * y) + EPS));
  double t3 = x * y * z * om::atan(y * z / (x * R + EPS));
  double t4 = 1.0 / 6.0 * (2 * x * x - y * y - z * z) * R;
  return t1 + t2 - t3 + t4;
}

// src/demag_cu.h:57-71
double newell_g(double x, double y, double z) {
  const double EPS = 1e-200;
  z = ABSV(z);
  double R = om::dsqrt(x * x + y * y + z * z);
  double t1 = x * y * z * om::asinh(z / (om::dsqrt(x * x + y * y) + EPS));
  double t2 = y / 6.0 * (3.0 * z * z - y * y) * om::asinh(x / (om::dsqrt(y * y + z * z) + EPS));
  double t3 = x / 6.0 * (3.0 * z * z - x * x) * om::asinh(y / (om::dsqrt(x * x + z * z) + EPS));
  double t4 = z * z * z / 6.0 * om::atan(x * y / (z * R + EPS));
  double t5 = z * y * y / 2.0 * om::atan(x * z / (y * R + EPS));
  double t6 = z * x * x / 2.0 * om::atan(y * z / (x * R + EPS));
  double t7 = x * y * R / 3.0;
  return t1 + t2 + t3 - t4 - t5 - t6 - t7;
}

// Offset wrap of src/demag_cu.cu:149-151.
int wrap_offset(int x, int n) { return (x + (n + 1) / 2 - 1) % n - (n + 1) / 2 + 1; }

// ktensorCPU (src/demag_cu.cu:119-248) for one padded point; out = xx,xy,xz,yy,yz,zz.
void newell_point(const Lat& L, double dx, double dy, double dz, double pi, int x, int y, int z,
                  double out[6], double far_r2 = 0.0) {
  int idx_x = wrap_offset(x, L.nxp), idx_y = wrap_offset(y, L.nyp), idx_z = wrap_offset(z, L.nzp);
  double kxx = 0, kxy = 0, kxz = 0, kyy = 0, kyz = 0, kzz = 0;
  for (int px = -L.P[0]; px <= L.P[0]; px++)
    for (int py = -L.P[1]; py <= L.P[1]; py++)
      for (int pz = -L.P[2]; pz <= L.P[2]; pz++) {
        int ix = idx_x + px * L.nxp, iy = idx_y + py * L.nyp, iz = idx_z + pz * L.nzp;
#ifndef ORACLE_LIBM
        if (far_r2 > 0.0) {  // far-field form of this image's 64 terms (newell_far.h)
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
#else
        (void)far_r2;
#endif
        for (int ikx = 0; ikx < 2; ikx++)
          for (int iky = 0; iky < 2; iky++)
            for (int ikz = 0; ikz < 2; ikz++)
              for (int ilx = 0; ilx < 2; ilx++)
                for (int ily = 0; ily < 2; ily++)
                  for (int ilz = 0; ilz < 2; ilz++) {
                    int iix = ix + ikx - ilx, iiy = iy + iky - ily, iiz = iz + ikz - ilz;
                    bool sign = ((ikx + iky + ikz + ilx + ily + ilz) % 2 == 0);
                    double X = iix * dx, Y = iiy * dy, Z = iiz * dz;
                    double t;
                    t = newell_f(X, Y, Z);
                    kxx += sign ? t : -t;
                    t = newell_g(X, Y, Z);
                    kxy += sign ? t : -t;
                    t = newell_g(X, Z, Y);
                    kxz += sign ? t : -t;
                    t = newell_f(Y, Z, X);
                    kyy += sign ? t : -t;
                    t = newell_g(Y, Z, X);
                    kyz += sign ? t : -t;
                    t = newell_f(Z, X, Y);
                    kzz += sign ? t : -t;
                  }
      }
  double d = -pi * 4.0 * dx * dy * dz;
  out[0] = kxx / d;
  out[1] = kxy / d;
  out[2] = kxz / d;
  out[3] = kyy / d;
  out[4] = kyz / d;
  out[5] = kzz / d;
}

// The same point with each image's 64 terms grouped by lattice node: the
// parity-signed sum over (ik, il) in {0,1}^2 per axis is, per axis, the
// weights 2 at s = ik - il = 0 and -1 at s = +-1, so an image's sum is
// sum_s w(sx) w(sy) w(sz) F(offset + s) over the 27 nodes s in {-1,0,1}^3
// (sx outer, sz inner; each product w F is exact, powers of two), formed per
// image and then added to the point's sum.  The GPU's node kernel evaluates F
// once per node and tile; this per-point form is its arithmetic.
void newell_point_nodes(const Lat& L, double dx, double dy, double dz, double pi, int x, int y, int z,
                        double out[6], double far_r2 = 0.0) {
  int idx_x = wrap_offset(x, L.nxp), idx_y = wrap_offset(y, L.nyp), idx_z = wrap_offset(z, L.nzp);
  double k[6] = {0, 0, 0, 0, 0, 0};
  const double w1[3] = {-1.0, 2.0, -1.0};
  for (int px = -L.P[0]; px <= L.P[0]; px++)
    for (int py = -L.P[1]; py <= L.P[1]; py++)
      for (int pz = -L.P[2]; pz <= L.P[2]; pz++) {
        int ix = idx_x + px * L.nxp, iy = idx_y + py * L.nyp, iz = idx_z + pz * L.nzp;
#ifndef ORACLE_LIBM
        if (far_r2 > 0.0) {
          const double X = ix * dx, Y = iy * dy, Z = iz * dz;
          if (X * X + Y * Y + Z * Z >= far_r2) {
            double r[6];
            mmcm::newell_far_raw(X, Y, Z, dx, dy, dz, r);
            for (int c = 0; c < 6; ++c) k[c] += r[c];
            continue;
          }
        }
#else
        (void)far_r2;
#endif
        double a[6] = {0, 0, 0, 0, 0, 0};
        for (int sx = -1; sx <= 1; ++sx)
          for (int sy = -1; sy <= 1; ++sy)
            for (int sz = -1; sz <= 1; ++sz) {
              const double w = w1[sx + 1] * w1[sy + 1] * w1[sz + 1];
              const double X = (ix + sx) * dx, Y = (iy + sy) * dy, Z = (iz + sz) * dz;
              a[0] += w * newell_f(X, Y, Z);
              a[1] += w * newell_g(X, Y, Z);
              a[2] += w * newell_g(X, Z, Y);
              a[3] += w * newell_f(Y, Z, X);
              a[4] += w * newell_g(Y, Z, X);
              a[5] += w * newell_f(Z, X, Y);
            }
        for (int c = 0; c < 6; ++c) k[c] += a[c];
      }
  const double d = -pi * 4.0 * dx * dy * dz;
  for (int c = 0; c < 6; ++c) out[c] = k[c] / d;
}

// ---------------------------------------------------------------- FFT
// Recursive mixed-radix decimation-in-time DFT (any length; prime factors
// handled by a direct sum).  sign = -1 forward, +1 inverse (unnormalised).
typedef std::complex<double> cd;

// Table of exp(sign 2 pi i e / n), e in [0, n), for the current length.
struct Roots {
  int n = 0, sign = 0;
  std::vector<cd> w;
  void make(int n_, int sign_) {
    if (n_ == n && sign_ == sign) return;
    n = n_;
    sign = sign_;
    w.resize(n);
    const double pi = 3.14159265358979323846;
    for (int e = 0; e < n; ++e) {
      double ang = sign * 2.0 * pi * (double)e / (double)n;
      w[e] = cd(std::cos(ang), std::sin(ang));
    }
  }
};

// e = r*kk reduced mod n through the table of the full length n: the roots of
// a sub-length m = n/s are every s-th entry.
void fft_rec(cd* x, int n, int stride, cd* out, const Roots& R, int rstep, cd* tmp) {
  if (n == 1) {
    out[0] = x[0];
    return;
  }
  int p = 2;
  while (n % p) ++p;
  int m = n / p;
  for (int r = 0; r < p; ++r) fft_rec(x + r * stride, m, stride * p, tmp + r * m, R, rstep * p, out);
  for (int k = 0; k < m; ++k)
    for (int q = 0; q < p; ++q) {
      int kk = k + q * m;
      cd s = tmp[k];
      for (int r = 1; r < p; ++r) {
        long e = ((long)r * kk) % n;
        s += tmp[r * m + k] * R.w[e * rstep];
      }
      out[kk] = s;
    }
}

void fft_inplace(cd* x, int n, int stride, int sign) {
  thread_local Roots R;
  thread_local std::vector<cd> a, o, t;
  R.make(n, sign);
  a.resize(n);
  o.resize(n);
  t.resize(n);
  for (int i = 0; i < n; ++i) a[i] = x[(long)i * stride];
  fft_rec(a.data(), n, 1, o.data(), R, 1, t.data());
  for (int i = 0; i < n; ++i) x[(long)i * stride] = o[i];
}

// 3-D transform of a padded grid (x fastest).
void fft3(std::vector<cd>& a, const Lat& L, int sign) {
  const int nx = L.nxp, ny = L.nyp, nz = L.nzp;
#pragma omp parallel for schedule(static)
  for (int r = 0; r < ny * nz; ++r) fft_inplace(a.data() + (long)r * nx, nx, 1, sign);
  if (ny > 1) {
#pragma omp parallel for schedule(static)
    for (int r = 0; r < nx * nz; ++r) {
      int x = r % nx, z = r / nx;
      fft_inplace(a.data() + (long)z * nx * ny + x, ny, nx, sign);
    }
  }
  if (nz > 1) {
#pragma omp parallel for schedule(static)
    for (int r = 0; r < nx * ny; ++r) fft_inplace(a.data() + r, nz, nx * ny, sign);
  }
}

struct DemagFFT {
  Lat L;
  std::vector<cd> K[6];
};

void demag_fft_prepare(DemagFFT& D, const Lat& L, const double* k6) {
  D.L = L;
  long np = L.np();
  for (int c = 0; c < 6; ++c) {
    D.K[c].assign(np, cd(0, 0));
    for (long i = 0; i < np; ++i) D.K[c][i] = cd(k6[c * np + i], 0.0);
    fft3(D.K[c], L, -1);
  }
}

// src/demag_cu.cu:68-116 (calHexchangeKernel): H^ = K^ . M^ / N for one
// frequency, K^ symmetric (xx, xy, xz, yy, yz, zz); each complex product is
// (a.x b.x - a.y b.y, a.x b.y + a.y b.x) and the three are summed left to right
// before the division, as there.
inline cd cmul(cd a, cd b) {
  return cd(a.real() * b.real() - a.imag() * b.imag(), a.real() * b.imag() + a.imag() * b.real());
}
inline void demag_product(cd mx, cd my, cd mz, const cd k[6], double N, cd h[3]) {
  const cd ax = cmul(mx, k[0]) + cmul(my, k[1]) + cmul(mz, k[2]);
  const cd ay = cmul(mx, k[1]) + cmul(my, k[3]) + cmul(mz, k[4]);
  const cd az = cmul(mx, k[2]) + cmul(my, k[4]) + cmul(mz, k[5]);
  h[0] = cd(ax.real() / N, ax.imag() / N);
  h[1] = cd(ay.real() / N, ay.imag() / N);
  h[2] = cd(az.real() / N, az.imag() / N);
}

// h = K * m (circular convolution on the padded grid, cropped), via full complex FFTs.
void demag_fft_apply(const DemagFFT& D, const double* m, double* h) {
  const Lat& L = D.L;
  long n = L.n(), np = L.np();
  std::vector<cd> M[3];
  for (int c = 0; c < 3; ++c) {
    M[c].assign(np, cd(0, 0));
    for (int z = 0; z < L.nz; ++z)
      for (int y = 0; y < L.ny; ++y)
        for (int x = 0; x < L.nx; ++x)
          M[c][x + (long)L.nxp * (y + (long)L.nyp * z)] = m[c * n + x + (long)L.nx * (y + (long)L.ny * z)];
    fft3(M[c], L, -1);
  }
  const double N = (double)np;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < np; ++i) {
    const cd k[6] = {D.K[0][i], D.K[1][i], D.K[2][i], D.K[3][i], D.K[4][i], D.K[5][i]};
    cd h[3];
    demag_product(M[0][i], M[1][i], M[2][i], k, N, h);
    M[0][i] = h[0];
    M[1][i] = h[1];
    M[2][i] = h[2];
  }
  for (int c = 0; c < 3; ++c) {
    fft3(M[c], L, +1);
    for (int z = 0; z < L.nz; ++z)
      for (int y = 0; y < L.ny; ++y)
        for (int x = 0; x < L.nx; ++x)
          h[c * n + x + (long)L.nx * (y + (long)L.ny * z)] = M[c][x + (long)L.nxp * (y + (long)L.nyp * z)].real();
  }
}

// ---------------------------------------------------------------- lattice helpers
// Neighbour of (x,y,z) along `axis` in direction dir (+1/-1), or -1 when the
// bond does not exist (open edge, or the wrapped neighbour is the cell itself).
long nbr(const Lat& L, int x, int y, int z, int axis, int dir) {
  int c[3] = {x, y, z};
  int n[3] = {L.nx, L.ny, L.nz};
  int v = c[axis] + dir;
  if (v < 0 || v >= n[axis]) {
    if (!L.per[axis]) return -1;
    v = (v + n[axis]) % n[axis];
  }
  if (v == c[axis]) return -1;
  c[axis] = v;
  return c[0] + (long)L.nx * (c[1] + (long)L.ny * c[2]);
}

int axis_color(int v, int n, bool per) {
  if (per && (n & 1) && n > 1 && v == n - 1) return 2;
  return v & 1;
}
int num_colors(const Lat& L) {
  int n[3] = {L.nx, L.ny, L.nz};
  for (int a = 0; a < 3; ++a)
    if (L.per[a] && (n[a] & 1) && n[a] > 1) return 3;
  return 2;
}
int cell_color(const Lat& L, int x, int y, int z) {
  int s = axis_color(x, L.nx, L.per[0]) + axis_color(y, L.ny, L.per[1]) + axis_color(z, L.nz, L.per[2]);
  return num_colors(L) == 2 ? (s & 1) : (s % 3);
}

struct Params {
  double V, ms, Aex, D, Ku1, u[3], B[3], mu0, d[3];
  bool demag;
};
Params params_of(const mmc_config* c) {
  Params p;
  p.d[0] = c->dx; p.d[1] = c->dy; p.d[2] = c->dz;
  p.V = c->dx * c->dy * c->dz;
  p.ms = c->ms; p.Aex = c->Aex; p.D = c->Dind; p.Ku1 = c->Ku1;
  double un = std::sqrt(c->anisUx * c->anisUx + c->anisUy * c->anisUy + c->anisUz * c->anisUz);
  p.u[0] = un > 0 ? c->anisUx / un : 0;
  p.u[1] = un > 0 ? c->anisUy / un : 0;
  p.u[2] = un > 0 ? c->anisUz / un : 0;
  p.B[0] = c->Bextx; p.B[1] = c->Bexty; p.B[2] = c->Bextz;
  p.mu0 = 4e-7 * pi_of(c);  // src/main.cu:244
  p.demag = c->cal_demag_flag != 0;
  return p;
}

}  // namespace

extern "C" {

int orc_padded_dims(const mmc_config* c, int out[3]) {
  Lat L = lat_of(c);
  out[0] = L.nxp;
  out[1] = L.nyp;
  out[2] = L.nzp;
  return 0;
}

double orc_newell_f(double x, double y, double z) { return newell_f(x, y, z); }
// Far-field form of the six 64-term sums of one image offset (newell_far.h).
void orc_newell_far(double X, double Y, double Z, double dx, double dy, double dz, double out[6]) {
#ifndef ORACLE_LIBM
  mmcm::newell_far_raw(X, Y, Z, dx, dy, dz, out);
#else
  (void)X, (void)Y, (void)Z, (void)dx, (void)dy, (void)dz;
  for (int k = 0; k < 6; ++k) out[k] = std::nan("");
#endif
}
// The exact six 64-term sums of one offset given in cells (before the -4 pi V division).
void orc_newell_raw(int ix, int iy, int iz, double dx, double dy, double dz, double out[6]) {
  double k[6] = {0, 0, 0, 0, 0, 0};
  for (int bits = 0; bits < 64; ++bits) {
    const int ikx = (bits >> 5) & 1, iky = (bits >> 4) & 1, ikz = (bits >> 3) & 1;
    const int ilx = (bits >> 2) & 1, ily = (bits >> 1) & 1, ilz = bits & 1;
    const bool sign = ((ikx + iky + ikz + ilx + ily + ilz) % 2 == 0);
    const double X = (ix + ikx - ilx) * dx, Y = (iy + iky - ily) * dy, Z = (iz + ikz - ilz) * dz;
    const double v[6] = {newell_f(X, Y, Z), newell_g(X, Y, Z), newell_g(X, Z, Y),
                         newell_f(Y, Z, X), newell_g(Y, Z, X), newell_f(Z, X, Y)};
    for (int c = 0; c < 6; ++c) k[c] += sign ? v[c] : -v[c];
  }
  for (int c = 0; c < 6; ++c) out[c] = k[c];
}
double orc_newell_g(double x, double y, double z) { return newell_g(x, y, z); }

void orc_math(int fn, const double* x, double* y, long n) {
  for (long i = 0; i < n; ++i) {
    double s, c;
    switch (fn) {
      case 0: y[i] = om::log(x[i]); break;
      case 1: y[i] = om::asinh(x[i]); break;
      case 2: y[i] = om::atan(x[i]); break;
      case 3: y[i] = om::exp(x[i]); break;
      case 4: om::sincospi(x[i], &s, &c); y[i] = s; break;
      case 5: om::sincospi(x[i], &s, &c); y[i] = c; break;
      default: y[i] = 0; break;
    }
  }
}

void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  om::u32x4 c = {ctr[0], ctr[1], ctr[2], ctr[3]};
  om::u32x4 r = om::philox4x32_10(c, key[0], key[1]);
  out[0] = r.x;
  out[1] = r.y;
  out[2] = r.z;
  out[3] = r.w;
}

// The frequency-domain product of demag_fft_apply on caller arrays: m3 holds
// three spectra of np complex values (interleaved re, im), k6 six, h3 three.
void orc_demag_product(long np, const double* m3, const double* k6, double* h3) {
  const cd* M = reinterpret_cast<const cd*>(m3);
  const cd* K = reinterpret_cast<const cd*>(k6);
  cd* H = reinterpret_cast<cd*>(h3);
  for (long i = 0; i < np; ++i) {
    const cd k[6] = {K[i], K[np + i], K[2 * np + i], K[3 * np + i], K[4 * np + i], K[5 * np + i]};
    cd h[3];
    demag_product(M[i], M[np + i], M[2 * np + i], k, (double)np, h);
    H[i] = h[0];
    H[np + i] = h[1];
    H[2 * np + i] = h[2];
  }
}

// The tensor at selected points of the padded grid (flat index x + nxp (y +
// nyp z)); out holds 6 blocks of `count` values.  The same per-point code as
// orc_newell_tensor, for checks of large lattices on a few points.
int orc_newell_points(const mmc_config* c, const long* idx, long count, double* out) {
#ifdef ORACLE_LIBM
  if (c->tensor_far_radius > 0) return -1;
#endif
  Lat L = lat_of(c);
  double pi = pi_of(c);
  double fr2 = 0.0;
  if (c->tensor_far_radius > 0) {
    const double d = std::max(c->dx, std::max(c->dy, c->dz)) * (double)c->tensor_far_radius;
    fr2 = d * d;
  }
#pragma omp parallel for schedule(dynamic)
  for (long j = 0; j < count; ++j) {
    const long i = idx[j];
    int x = (int)(i % L.nxp), y = (int)((i / L.nxp) % L.nyp), z = (int)(i / ((long)L.nxp * L.nyp));
    double o[6];
    if (c->tensor_sum == 1) newell_point_nodes(L, c->dx, c->dy, c->dz, pi, x, y, z, o, fr2);
    else newell_point(L, c->dx, c->dy, c->dz, pi, x, y, z, o, fr2);
    for (int k = 0; k < 6; ++k) out[k * count + j] = o[k];
  }
  return 0;
}

// Full tensor, 6 blocks of nxp*nyp*nzp doubles (x fastest).
int orc_newell_tensor(const mmc_config* c, double* k6) {
#ifdef ORACLE_LIBM
  if (c->tensor_far_radius > 0) return -1;  // the far-field form is not in the independent build
#endif
  Lat L = lat_of(c);
  long np = L.np();
  double pi = pi_of(c);
#pragma omp parallel for schedule(dynamic)
  for (long i = 0; i < np; ++i) {
    int x = (int)(i % L.nxp), y = (int)((i / L.nxp) % L.nyp), z = (int)(i / ((long)L.nxp * L.nyp));
    double o[6];
    double fr2 = 0.0;
    if (c->tensor_far_radius > 0) {
      const double d = std::max(c->dx, std::max(c->dy, c->dz)) * (double)c->tensor_far_radius;
      fr2 = d * d;
    }
    if (c->tensor_sum == 1) newell_point_nodes(L, c->dx, c->dy, c->dz, pi, x, y, z, o, fr2);
    else newell_point(L, c->dx, c->dy, c->dz, pi, x, y, z, o, fr2);
    for (int k = 0; k < 6; ++k) k6[k * np + i] = o[k];
  }
  return 0;
}

// Uniform random unit vectors keyed on (seed, cell) -- stream STREAM_INIT.
void orc_init_random(const mmc_config* c, long long seed, double* m) {
  Lat L = lat_of(c);
  long n = L.n();
  uint32_t k0 = (uint32_t)((uint64_t)seed & 0xffffffffu), k1 = (uint32_t)((uint64_t)seed >> 32);
  for (long i = 0; i < n; ++i) {
    om::u32x4 ctr = {(uint32_t)i, 0u, 0u, om::STREAM_INIT};
    om::u32x4 r = om::philox4x32_10(ctr, k0, k1);
    double z = 2.0 * om::u01_f64(r.x) - 1.0;
    double t = 1.0 - z * z;
    if (t < 0) t = 0;
    double s = om::dsqrt(t), sn, cs;
    om::sincospi(2.0 * om::u01_f64(r.y), &sn, &cs);
    m[i] = s * cs;
    m[n + i] = s * sn;
    m[2 * n + i] = z;
  }
}

// Direct O(N^2) circular convolution on the padded grid (independent of any FFT).
int orc_demag_direct(const mmc_config* c, const double* k6, const double* m, double* h) {
  Lat L = lat_of(c);
  long n = L.n(), np = L.np();
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) {
    int xi = (int)(i % L.nx), yi = (int)((i / L.nx) % L.ny), zi = (int)(i / ((long)L.nx * L.ny));
    double hx = 0, hy = 0, hz = 0;
    for (long j = 0; j < n; ++j) {
      int xj = (int)(j % L.nx), yj = (int)((j / L.nx) % L.ny), zj = (int)(j / ((long)L.nx * L.ny));
      int ox = ((xi - xj) % L.nxp + L.nxp) % L.nxp;
      int oy = ((yi - yj) % L.nyp + L.nyp) % L.nyp;
      int oz = ((zi - zj) % L.nzp + L.nzp) % L.nzp;
      long o = ox + (long)L.nxp * (oy + (long)L.nyp * oz);
      double mx = m[j], my = m[n + j], mz = m[2 * n + j];
      double xx = k6[o], xy = k6[np + o], xz = k6[2 * np + o], yy = k6[3 * np + o], yz = k6[4 * np + o],
             zz = k6[5 * np + o];
      hx += xx * mx + xy * my + xz * mz;
      hy += xy * mx + yy * my + yz * mz;
      hz += xz * mx + yz * my + zz * mz;
    }
    h[i] = hx;
    h[n + i] = hy;
    h[2 * n + i] = hz;
  }
  return 0;
}

int orc_demag_fft(const mmc_config* c, const double* k6, const double* m, double* h) {
  DemagFFT D;
  demag_fft_prepare(D, lat_of(c), k6);
  demag_fft_apply(D, m, h);
  return 0;
}

// Effective field of one term in A/m.  hd is the dimensionless demag field
// h = K * m (so H_demag = Ms h).
int orc_field(const mmc_config* c, int term, const double* m, const double* hd, double* H) {
  Lat L = lat_of(c);
  Params p = params_of(c);
  long n = L.n();
  const double* mx = m;
  const double* my = m + n;
  const double* mz = m + 2 * n;
  for (int z = 0; z < L.nz; ++z)
    for (int y = 0; y < L.ny; ++y)
      for (int x = 0; x < L.nx; ++x) {
        long i = x + (long)L.nx * (y + (long)L.ny * z);
        double f[3] = {0, 0, 0};
        if (term == MMC_TERM_EXCHANGE || term == MMC_TERM_TOTAL) {
          double pre = 2.0 * p.Aex / (p.mu0 * p.ms);
          for (int a = 0; a < 3; ++a)
            for (int dir = -1; dir <= 1; dir += 2) {
              long j = nbr(L, x, y, z, a, dir);
              if (j < 0) continue;
              double w = pre / (p.d[a] * p.d[a]);
              f[0] += w * (mx[j] - mx[i]);
              f[1] += w * (my[j] - my[i]);
              f[2] += w * (mz[j] - mz[i]);
            }
        }
        if (term == MMC_TERM_DMI || term == MMC_TERM_TOTAL) {
          double pre = 2.0 * p.D / (p.mu0 * p.ms);
          long xp = nbr(L, x, y, z, 0, 1), xm = nbr(L, x, y, z, 0, -1);
          long yp = nbr(L, x, y, z, 1, 1), ym = nbr(L, x, y, z, 1, -1);
          double dxmz = ((xp >= 0 ? mz[xp] : 0.0) - (xm >= 0 ? mz[xm] : 0.0)) / (2.0 * p.d[0]);
          double dxmx = ((xp >= 0 ? mx[xp] : 0.0) - (xm >= 0 ? mx[xm] : 0.0)) / (2.0 * p.d[0]);
          double dymz = ((yp >= 0 ? mz[yp] : 0.0) - (ym >= 0 ? mz[ym] : 0.0)) / (2.0 * p.d[1]);
          double dymy = ((yp >= 0 ? my[yp] : 0.0) - (ym >= 0 ? my[ym] : 0.0)) / (2.0 * p.d[1]);
          f[0] += pre * dxmz;
          f[1] += pre * dymz;
          f[2] += pre * (-dxmx - dymy);
        }
        if (term == MMC_TERM_ANISOTROPY || term == MMC_TERM_TOTAL) {
          double pre = 2.0 * p.Ku1 / (p.mu0 * p.ms);
          double mu = mx[i] * p.u[0] + my[i] * p.u[1] + mz[i] * p.u[2];
          for (int k = 0; k < 3; ++k) f[k] += pre * mu * p.u[k];
        }
        if (term == MMC_TERM_ZEEMAN || term == MMC_TERM_TOTAL) {
          for (int k = 0; k < 3; ++k) f[k] += p.B[k] / p.mu0;
        }
        if ((term == MMC_TERM_DEMAG || term == MMC_TERM_TOTAL) && p.demag && hd) {
          for (int k = 0; k < 3; ++k) f[k] += p.ms * hd[k * n + i];
        }
        H[i] = f[0];
        H[n + i] = f[1];
        H[2 * n + i] = f[2];
      }
  return 0;
}

// Energies (J) and observables of m.  out: [E_ex, E_dmi, E_an, E_zeeman, E_demag,
// <mx>, <my>, <mz>, Q].
int orc_energy(const mmc_config* c, const double* m, const double* hd, double out[9]) {
  Lat L = lat_of(c);
  Params p = params_of(c);
  long n = L.n();
  const double* mx = m;
  const double* my = m + n;
  const double* mz = m + 2 * n;
  double eex = 0, edm = 0, ean = 0, ez = 0, ed = 0, sx = 0, sy = 0, sz = 0, q = 0;
  for (int z = 0; z < L.nz; ++z)
    for (int y = 0; y < L.ny; ++y)
      for (int x = 0; x < L.nx; ++x) {
        long i = x + (long)L.nx * (y + (long)L.ny * z);
        for (int a = 0; a < 3; ++a) {
          long j = nbr(L, x, y, z, a, 1);
          if (j < 0) continue;
          double ddx = mx[j] - mx[i], ddy = my[j] - my[i], ddz = mz[j] - mz[i];
          eex += p.Aex * p.V * (ddx * ddx + ddy * ddy + ddz * ddz) / (p.d[a] * p.d[a]);
        }
        long xp = nbr(L, x, y, z, 0, 1), xm = nbr(L, x, y, z, 0, -1);
        long yp = nbr(L, x, y, z, 1, 1), ym = nbr(L, x, y, z, 1, -1);
        double dxmz = ((xp >= 0 ? mz[xp] : 0.0) - (xm >= 0 ? mz[xm] : 0.0)) / (2.0 * p.d[0]);
        double dxmx = ((xp >= 0 ? mx[xp] : 0.0) - (xm >= 0 ? mx[xm] : 0.0)) / (2.0 * p.d[0]);
        double dymz = ((yp >= 0 ? mz[yp] : 0.0) - (ym >= 0 ? mz[ym] : 0.0)) / (2.0 * p.d[1]);
        double dymy = ((yp >= 0 ? my[yp] : 0.0) - (ym >= 0 ? my[ym] : 0.0)) / (2.0 * p.d[1]);
        edm += -p.D * p.V * (mx[i] * dxmz + my[i] * dymz + mz[i] * (-dxmx - dymy));
        double mu = mx[i] * p.u[0] + my[i] * p.u[1] + mz[i] * p.u[2];
        ean += -p.Ku1 * p.V * mu * mu;
        ez += -p.ms * p.V * (mx[i] * p.B[0] + my[i] * p.B[1] + mz[i] * p.B[2]);
        if (p.demag && hd)
          ed += -0.5 * p.mu0 * p.ms * p.ms * p.V * (mx[i] * hd[i] + my[i] * hd[n + i] + mz[i] * hd[2 * n + i]);
        sx += mx[i];
        sy += my[i];
        sz += mz[i];
        // Berg-Luescher topological charge of the plaquette with (x,y) as lower-left corner.
        long i2 = nbr(L, x, y, z, 0, 1);
        long i4 = nbr(L, x, y, z, 1, 1);
        if (i2 >= 0 && i4 >= 0) {
          int x2 = (int)(i2 % L.nx);
          long i3 = nbr(L, x2, y, z, 1, 1);
          long tri[2][3] = {{i, i2, i3}, {i, i3, i4}};
          for (int t = 0; t < 2; ++t) {
            long a = tri[t][0], b = tri[t][1], cc = tri[t][2];
            double ax = mx[a], ay = my[a], az = mz[a];
            double bx = mx[b], by = my[b], bz = mz[b];
            double cx = mx[cc], cy = my[cc], cz = mz[cc];
            double trip = ax * (by * cz - bz * cy) + ay * (bz * cx - bx * cz) + az * (bx * cy - by * cx);
            double den = 1.0 + (ax * bx + ay * by + az * bz) + (bx * cx + by * cy + bz * cz) +
                         (cx * ax + cy * ay + cz * az);
            q += 2.0 * std::atan2(trip, den);
          }
        }
      }
  const double pi = 3.14159265358979323846;
  out[0] = eex;
  out[1] = edm;
  out[2] = ean;
  out[3] = ez;
  out[4] = ed;
  out[5] = sx / (double)n;
  out[6] = sy / (double)n;
  out[7] = sz / (double)n;
  out[8] = q / (4.0 * pi) / (double)L.nz;
  return 0;
}

// Metropolis sweeps: per sweep, one demag refresh (if enabled), then every
// sublattice colour in turn; each cell of the colour draws
// Philox(seed; cell, sweep, stage, 0) -> (u0, u1, u2), proposes
// m' = (sqrt(1-z^2) cos 2 pi u1, sqrt(1-z^2) sin 2 pi u1, z = 2 u0 - 1) and
// accepts when dE <= 0 or u2 < exp(-dE/kT).
// demag_mode: 0 = direct sum, 1 = FFT.  nthreads <= 0 keeps the OpenMP default.
int orc_sweeps(const mmc_config* c, const double* k6, double T, long long stage, long long sweep0,
               long long nsweeps, double* m, unsigned long long* accepted, int demag_mode,
               int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  Lat L = lat_of(c);
  Params p = params_of(c);
  long n = L.n(), np = L.np();
  double* mx = m;
  double* my = m + n;
  double* mz = m + 2 * n;
  const double kT = kB * T;
  double wex[3];
  for (int a = 0; a < 3; ++a) wex[a] = 2.0 * p.Aex * p.V / (p.d[a] * p.d[a] * kT);
  double wdm0 = p.D * p.V / (p.d[0] * kT), wdm1 = p.D * p.V / (p.d[1] * kT);
  double can = p.Ku1 * p.V / kT;
  double czx = p.ms * p.V * p.B[0] / kT, czy = p.ms * p.V * p.B[1] / kT, czz = p.ms * p.V * p.B[2] / kT;
  double cd = p.demag ? p.mu0 * p.ms * p.ms * p.V / kT : 0.0;
  double k0[6] = {0, 0, 0, 0, 0, 0};
  if (p.demag)
    for (int k = 0; k < 6; ++k) k0[k] = k6[k * np];
  std::vector<double> h(p.demag ? 3 * n : 0);
  DemagFFT D;
  if (p.demag && demag_mode == 1) demag_fft_prepare(D, L, k6);
  uint32_t key0 = (uint32_t)((uint64_t)c->randomseed & 0xffffffffu), key1 = (uint32_t)((uint64_t)c->randomseed >> 32);
  const int ncol = num_colors(L);
  unsigned long long acc = 0;
  for (long long s = 0; s < nsweeps; ++s) {
    uint32_t sweep = (uint32_t)(sweep0 + s);
    if (p.demag) {
      if (demag_mode == 1) demag_fft_apply(D, m, h.data());
      else orc_demag_direct(c, k6, m, h.data());
    }
    for (int col = 0; col < ncol; ++col) {
#pragma omp parallel for schedule(static) reduction(+ : acc)
      for (long i = 0; i < n; ++i) {
        int x = (int)(i % L.nx), y = (int)((i / L.nx) % L.ny), z = (int)(i / ((long)L.nx * L.ny));
        if (cell_color(L, x, y, z) != col) continue;
        double Fx = 0, Fy = 0, Fz = 0;
        long nb[3][2];
        for (int a = 0; a < 3; ++a) {
          nb[a][0] = nbr(L, x, y, z, a, -1);
          nb[a][1] = nbr(L, x, y, z, a, 1);
          for (int s2 = 0; s2 < 2; ++s2) {
            long j = nb[a][s2];
            if (j < 0) continue;
            Fx = Fx + wex[a] * mx[j];
            Fy = Fy + wex[a] * my[j];
            Fz = Fz + wex[a] * mz[j];
          }
        }
        long xm = nb[0][0], xp = nb[0][1], ym = nb[1][0], yp = nb[1][1];
        double dxmz = (xp >= 0 ? mz[xp] : 0.0) - (xm >= 0 ? mz[xm] : 0.0);
        double dxmx = (xp >= 0 ? mx[xp] : 0.0) - (xm >= 0 ? mx[xm] : 0.0);
        double dymz = (yp >= 0 ? mz[yp] : 0.0) - (ym >= 0 ? mz[ym] : 0.0);
        double dymy = (yp >= 0 ? my[yp] : 0.0) - (ym >= 0 ? my[ym] : 0.0);
        Fx = Fx + wdm0 * dxmz;
        Fy = Fy + wdm1 * dymz;
        Fz = Fz - (wdm0 * dxmx + wdm1 * dymy);
        Fx = Fx + czx;
        Fy = Fy + czy;
        Fz = Fz + czz;
        double ox = mx[i], oy = my[i], oz = mz[i];
        if (cd != 0.0) {
          double sx = k0[0] * ox + k0[1] * oy + k0[2] * oz;
          double sy = k0[1] * ox + k0[3] * oy + k0[4] * oz;
          double sz = k0[2] * ox + k0[4] * oy + k0[5] * oz;
          Fx = Fx + cd * (h[i] - sx);
          Fy = Fy + cd * (h[n + i] - sy);
          Fz = Fz + cd * (h[2 * n + i] - sz);
        }
        om::u32x4 ctr = {(uint32_t)i, sweep, (uint32_t)stage, om::STREAM_SWEEP};
        om::u32x4 r = om::philox4x32_10(ctr, key0, key1);
        double pz = 2.0 * om::u01_f64(r.x) - 1.0;
        double t = 1.0 - pz * pz;
        if (t < 0) t = 0;
        double st = om::dsqrt(t), sn, cs;
        om::sincospi(2.0 * om::u01_f64(r.y), &sn, &cs);
        double px = st * cs, py = st * sn;
        double ddx = px - ox, ddy = py - oy, ddz = pz - oz;
        double dE = -(ddx * Fx + ddy * Fy + ddz * Fz);
        double pun = px * p.u[0] + py * p.u[1] + pz * p.u[2];
        double puo = ox * p.u[0] + oy * p.u[1] + oz * p.u[2];
        dE = dE - can * (pun * pun - puo * puo);
        if (cd != 0.0) {
          double qn = px * (k0[0] * px + k0[1] * py + k0[2] * pz) + py * (k0[1] * px + k0[3] * py + k0[4] * pz) +
                      pz * (k0[2] * px + k0[4] * py + k0[5] * pz);
          double qo = ox * (k0[0] * ox + k0[1] * oy + k0[2] * oz) + oy * (k0[1] * ox + k0[3] * oy + k0[4] * oz) +
                      oz * (k0[2] * ox + k0[4] * oy + k0[5] * oz);
          dE = dE - 0.5 * cd * (qn - qo);
        }
        double u2 = om::u01_f64(r.z);
        if (dE <= 0.0 || u2 < om::exp(-dE)) {
          mx[i] = px;
          my[i] = py;
          mz[i] = pz;
          acc += 1;
        }
      }
    }
  }
  if (accepted) *accepted = acc;
  return 0;
}

// Local energy change of proposing m' at cell i, in J, from the global energy
// difference (used to test the local formula).
double orc_energy_total(const mmc_config* c, const double* m, const double* hd) {
  double o[9];
  orc_energy(c, m, hd, o);
  return o[0] + o[1] + o[2] + o[3] + o[4];
}


// Gradient of the total energy (orc_energy's five terms) with respect to m,
// treating the three components of every cell as free variables, and with
// respect to the scalars (Aex, Dind, Ku1, Ms, Bx, By, Bz).  The bilinear
// exchange and DMI energies have symmetric operators and Zeeman/anisotropy are
// local, so dE/dm_i = -mu0 Ms V H_i for those terms.  The demag energy
// -mu0 Ms^2 V/2 sum m.(K*m) has gradient -mu0 Ms^2 V/2 (K*m + K'*m) with
// K'(r) = K(-r); K' differs from K only through the far periodic image on even
// axes, and both are convolved here.  grad: 3n doubles (may be NULL);
// dparams: 7 doubles.
int orc_grad(const mmc_config* c, const double* k6, const double* m, double* grad, double dparams[7]) {
  Lat L = lat_of(c);
  Params p = params_of(c);
  const long n = L.n(), np = L.np();
  std::vector<double> hs;
  if (p.demag) {
    if (!k6) return 1;
    std::vector<double> h(3 * n), h2(3 * n), kr(6 * np);
    // K'(x, y, z) = K(-x, -y, -z) on the padded grid
    for (int z = 0; z < L.nzp; ++z)
      for (int y = 0; y < L.nyp; ++y)
        for (int x = 0; x < L.nxp; ++x) {
          const long o = x + (long)L.nxp * (y + (long)L.nyp * z);
          const long r = (L.nxp - x) % L.nxp + (long)L.nxp * ((L.nyp - y) % L.nyp + (long)L.nyp * ((L.nzp - z) % L.nzp));
          for (int k = 0; k < 6; ++k) kr[k * np + o] = k6[k * np + r];
        }
    orc_demag_fft(c, k6, m, h.data());
    orc_demag_fft(c, kr.data(), m, h2.data());
    hs.resize(3 * n);
    for (long i = 0; i < 3 * n; ++i) hs[i] = 0.5 * (h[i] + h2[i]);
  }
  if (grad) {
    std::vector<double> H(3 * n);
    orc_field(c, MMC_TERM_TOTAL, m, p.demag ? hs.data() : nullptr, H.data());
    const double s = -p.mu0 * p.ms * p.V;
    for (long i = 0; i < 3 * n; ++i) grad[i] = s * H[i];
  }
  // the energy is linear in Aex, Dind and Ku1: their derivatives are the
  // energies at unit strength
  mmc_config u = *c;
  u.Aex = 1.0;
  u.Dind = 1.0;
  u.Ku1 = 1.0;
  double eu[9], e[9];
  orc_energy(&u, m, p.demag ? hs.data() : nullptr, eu);
  orc_energy(c, m, p.demag ? hs.data() : nullptr, e);
  dparams[0] = eu[0];
  dparams[1] = eu[1];
  dparams[2] = eu[2];
  // Zeeman is linear and demag quadratic in Ms
  dparams[3] = (e[3] + 2.0 * e[4]) / p.ms;
  for (int k = 0; k < 3; ++k) dparams[4 + k] = -p.ms * p.V * e[5 + k] * (double)n;
  return 0;
}

}  // extern "C"
