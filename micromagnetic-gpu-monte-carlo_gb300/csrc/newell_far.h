// newell_far.h -- far-field expansion of the Newell tensor sums, compiled
// identically for the host (oracle) and the device (k_newell).
//
// The tensor sum of one image offset r = (X, Y, Z) is a second central
// difference in each axis of Newell's f (diagonal) or g (off-diagonal),
// K_ab = Dx^2 Dy^2 Dz^2 F / (4 pi V).  With D_h^2 = h^2 d^2 (1 + h^2 d^2 / 12 +
// h^4 d^4 / 360 + h^6 d^6 / 20160 + ...) (the Taylor series of a central
// second difference) and d_x^2 d_y^2 d_z^2 f = d_x^2 (1/R),
// d_x^2 d_y^2 d_z^2 g = d_x d_y (1/R), the sum becomes
//   K_ab = V / (4 pi) * P(d) d_a d_b (1/R),
//   P = prod_c (1 + h_c^2 d_c^2 / 12 + h_c^4 d_c^4 / 360 + h_c^6 d_c^6 / 20160),
// truncated here after the terms of total derivative order 6 on top of
// d_a d_b, so the relative error is O((h/R)^8): below 1e-11 beyond 20 cells
// and 1e-13 beyond 40.  The exact 64-term sum loses about (R/h)^6 x 1e-16 to
// cancellation there, so beyond a few tens of cells this form is the more
// accurate one.  The derivatives of 1/R come from the recurrence of its Taylor
// coefficients a_k = d^k (1/R) / k! (multi-index k, |k| = n):
//   n R^2 a_k = -(2n - 1) sum_i x_i a_{k - e_i} - (n - 1) sum_i a_{k - 2 e_i}.
// No counterpart in the reference, which sums every image exactly
// (src/demag_cu.cu:119-248).
#pragma once
#include "mmc_math.h"

namespace mmcm {

constexpr int NF_ORDER = 8;   // largest derivative order needed
constexpr int NF_COUNT = 165;  // multi-indices with |k| <= 8

// Position of multi-index (kx, ky, kz) in the table: orders are stored one
// after the other, and within order n by m = ky + kz, then kz.
MMC_HD int nf_index(int kx, int ky, int kz) {
  const int n = kx + ky + kz, m = ky + kz;
  return n * (n + 1) * (n + 2) / 6 + m * (m + 1) / 2 + kz;
}

MMC_HD double nf_fact(int k) {
  double f = 1.0;
  for (int i = 2; i <= k; ++i) f *= (double)i;
  return f;
}

// d^(kx,ky,kz) (1/R) from the coefficient table.
MMC_HD double nf_deriv(const double* a, int kx, int ky, int kz) {
  return nf_fact(kx) * nf_fact(ky) * nf_fact(kz) * a[nf_index(kx, ky, kz)];
}

// Taylor coefficients of 1/R at (x, y, z) up to order NF_ORDER.
MMC_HD void nf_coefficients(double x, double y, double z, double* a) {
  const double R2 = x * x + y * y + z * z;
  a[0] = 1.0 / dsqrt(R2);
  for (int n = 1; n <= NF_ORDER; ++n)
    for (int m = 0; m <= n; ++m)
      for (int kz = 0; kz <= m; ++kz) {
        const int ky = m - kz, kx = n - m;
        double s1 = 0.0, s2 = 0.0;
        if (kx >= 1) s1 = s1 + x * a[nf_index(kx - 1, ky, kz)];
        if (ky >= 1) s1 = s1 + y * a[nf_index(kx, ky - 1, kz)];
        if (kz >= 1) s1 = s1 + z * a[nf_index(kx, ky, kz - 1)];
        if (kx >= 2) s2 = s2 + a[nf_index(kx - 2, ky, kz)];
        if (ky >= 2) s2 = s2 + a[nf_index(kx, ky - 2, kz)];
        if (kz >= 2) s2 = s2 + a[nf_index(kx, ky, kz - 2)];
        a[nf_index(kx, ky, kz)] = -((double)(2 * n - 1) * s1 + (double)(n - 1) * s2) / ((double)n * R2);
      }
}

// P(d) d^b (1/R) for the base multi-index b (|b| = 2).
MMC_HD double nf_series(const double* a, const int b[3], const double h[3]) {
  double h2[3], h4[3], h6[3];
  for (int c = 0; c < 3; ++c) {
    h2[c] = h[c] * h[c];
    h4[c] = h2[c] * h2[c];
    h6[c] = h4[c] * h2[c];
  }
  double s = nf_deriv(a, b[0], b[1], b[2]);
  // single-axis terms of orders 2, 4, 6
  for (int c = 0; c < 3; ++c) {
    int k[3] = {b[0], b[1], b[2]};
    k[c] += 2;
    s = s + h2[c] / 12.0 * nf_deriv(a, k[0], k[1], k[2]);
    k[c] += 2;
    s = s + h4[c] / 360.0 * nf_deriv(a, k[0], k[1], k[2]);
    k[c] += 2;
    s = s + h6[c] / 20160.0 * nf_deriv(a, k[0], k[1], k[2]);
  }
  // two-axis terms of orders 4 (2+2) and 6 (4+2)
  for (int c = 0; c < 3; ++c)
    for (int d = 0; d < 3; ++d) {
      if (d == c) continue;
      int k[3] = {b[0], b[1], b[2]};
      k[c] += 4;
      k[d] += 2;
      s = s + h4[c] * h2[d] / 4320.0 * nf_deriv(a, k[0], k[1], k[2]);
      if (c < d) {
        int q[3] = {b[0], b[1], b[2]};
        q[c] += 2;
        q[d] += 2;
        s = s + h2[c] * h2[d] / 144.0 * nf_deriv(a, q[0], q[1], q[2]);
      }
    }
  // three-axis term of order 6
  {
    const int k[3] = {b[0] + 2, b[1] + 2, b[2] + 2};
    s = s + h2[0] * h2[1] * h2[2] / 1728.0 * nf_deriv(a, k[0], k[1], k[2]);
  }
  return s;
}

// The six 64-term sums (xx, xy, xz, yy, yz, zz) of one image offset, in the
// units of the exact sums before their division by -4 pi V:
// raw_ab = -V^2 P d_a d_b (1/R).
MMC_HD void newell_far_raw(double X, double Y, double Z, double dx, double dy, double dz, double out[6]) {
  double a[NF_COUNT];
  nf_coefficients(X, Y, Z, a);
  const double h[3] = {dx, dy, dz};
  const double V = dx * dy * dz;
  const int base[6][3] = {{2, 0, 0}, {1, 1, 0}, {1, 0, 1}, {0, 2, 0}, {0, 1, 1}, {0, 0, 2}};
  for (int c = 0; c < 6; ++c) out[c] = -(V * V) * nf_series(a, base[c], h);
}

}  // namespace mmcm
