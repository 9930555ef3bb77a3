// coef.h -- Metropolis coefficients from the material parameters and T.
//
// One function, compiled for the host runtime (g++ -ffp-contract=off) and for
// the device swap kernel (nvcc -fmad=false), so that a replica whose
// temperature changes on the device gets bit-for-bit the coefficients the host
// would have computed.
#pragma once
#include "mmc_internal.h"

namespace mmc {

// Temperature-independent inputs of McCoef (SI).
struct McParams {
  double aex, dind, ku1, ms;
  double b[3];
  double u[3];     // normalised anisotropy axis
  double d[3];
  double v;        // dx dy dz
  double mu0;
  double k0[6];    // self tensor (0 when demag is off)
  int demag;
  uint32_t key0, key1;
};

#if defined(__CUDACC__)
#define MMC_COEF_HD __host__ __device__
#else
#define MMC_COEF_HD
#endif

template <typename T>
MMC_COEF_HD inline McCoef<T> mc_coef_from(const McParams& p, double T_K) {
  const double kB = 1.3806488e-23;  // src/constant.h:22
  const double kT = kB * T_K;
  McCoef<T> k;
  for (int a = 0; a < 3; ++a) k.wex[a] = (T)(2.0 * p.aex * p.v / (p.d[a] * p.d[a] * kT));
  k.wdm[0] = (T)(p.dind * p.v / (p.d[0] * kT));
  k.wdm[1] = (T)(p.dind * p.v / (p.d[1] * kT));
  k.can = (T)(p.ku1 * p.v / kT);
  for (int a = 0; a < 3; ++a) k.u[a] = (T)p.u[a];
  k.cz[0] = (T)(p.ms * p.v * p.b[0] / kT);
  k.cz[1] = (T)(p.ms * p.v * p.b[1] / kT);
  k.cz[2] = (T)(p.ms * p.v * p.b[2] / kT);
  k.cd = (T)(p.demag ? p.mu0 * p.ms * p.ms * p.v / kT : 0.0);
  for (int q = 0; q < 6; ++q) k.k0[q] = (T)(p.demag ? p.k0[q] : 0.0);
  for (int q = 0; q < 6; ++q) k.k0h[q] = (T)(p.demag ? 0.5 * (p.mu0 * p.ms * p.ms * p.v / kT) * p.k0[q] : 0.0);
  k.key0 = p.key0;
  k.key1 = p.key1;
  return k;
}

}  // namespace mmc
