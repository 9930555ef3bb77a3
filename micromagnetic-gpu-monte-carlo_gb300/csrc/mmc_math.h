// mmc_math.h -- deterministic FP64 elementary functions and the Philox4x32-10
// counter-based generator, compiled identically for the host (g++) and the
// device (nvcc).
//
// Why this exists: the Newell demag tensor (reference src/demag_cu.h:43-71,
// src/demag_cu.cu:119-248) is a 64-term alternating sum of asinh/atan/sqrt
// terms whose magnitude grows like r^3 while the result decays like r^-3, so
// for far periodic images the result is dominated by rounding.  Two builds of
// that sum only agree if they evaluate every elementary function with the
// same operation sequence.  The functions below are written from their
// mathematical definitions (argument reduction + Taylor / atanh series whose
// coefficients are 1/n!, 1/(2k+1)), not from any vendor math library, and use
// only +,-,*,/ and IEEE sqrt, which are correctly rounded on both the CPU and
// the GPU.  Translation units that use them in FP64 must be compiled without
// multiply-add contraction (nvcc -fmad=false, gcc -ffp-contract=off) so the
// host and device produce bit-identical results.
//
// Philox4x32-10 follows J. K. Salmon, M. A. Moraes, R. O. Dror, D. E. Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11 (multipliers
// 0xD2511F53 / 0xCD9E8D57, Weyl key increments 0x9E3779B9 / 0xBB67AE85).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define MMC_HD __host__ __device__ __forceinline__
#else
#define MMC_HD static inline
#endif

#if !defined(__CUDA_ARCH__)
#include <string.h>
#include <math.h>
#endif

namespace mmcm {

// ---------------------------------------------------------------- bit helpers
MMC_HD uint64_t dbits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
#endif
}

MMC_HD double bitsd(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, 8);
  return x;
#endif
}

// IEEE-754 round-to-nearest square root on both sides.
MMC_HD double dsqrt(double x) {
#if defined(__CUDA_ARCH__)
  return __dsqrt_rn(x);
#else
  return sqrt(x);
#endif
}

MMC_HD double dfloor(double x) {
#if defined(__CUDA_ARCH__)
  return floor(x);
#else
  return floor(x);
#endif
}

MMC_HD double dabs(double x) { return x < 0.0 ? -x : x; }

// ln 2 split so that k*LN2_HI is exact for |k| < 2^21.
#define MMCM_LN2_HI 0x1.62e42ff000000p-1
#define MMCM_LN2_LO -0x1.718432a1b0e26p-35
#define MMCM_LN2 0x1.62e42fefa39efp-1
#define MMCM_INV_LN2 0x1.71547652b82fep+0
#define MMCM_SQRT2 0x1.6a09e667f3bcdp+0
#define MMCM_PI_HI 0x1.921fb54442d18p+1
#define MMCM_PI_LO 0x1.1a62633145c07p-53
#define MMCM_PIO2_HI 0x1.921fb54442d18p+0
#define MMCM_PIO2_LO 0x1.1a62633145c07p-54
#define MMCM_PIO4_HI 0x1.921fb54442d18p-1
#define MMCM_PIO4_LO 0x1.1a62633145c07p-55
#define MMCM_ATAN_HALF_HI 0x1.dac670561bb4fp-2
#define MMCM_ATAN_HALF_LO 0x1.a2b7f222f65e2p-56
#define MMCM_ATAN_3HALF_HI 0x1.f730bd281f69bp-1
#define MMCM_ATAN_3HALF_LO 0x1.007887af0cbbdp-56

// 2*atanh(s)/ (2s) = sum_k s^(2k) / (2k+1), evaluated by Horner in w = s^2.
// |s| <= 0.1716 here, so 12 terms leave a truncation error below 2^-60.
MMC_HD double atanh_series(double w) {
  double p = 0x1.642c8590b2164p-5;  // 1/23
  p = p * w + 0x1.8618618618618p-5; // 1/21
  p = p * w + 0x1.af286bca1af28p-5; // 1/19
  p = p * w + 0x1.e1e1e1e1e1e1ep-5; // 1/17
  p = p * w + 0x1.1111111111111p-4; // 1/15
  p = p * w + 0x1.3b13b13b13b14p-4; // 1/13
  p = p * w + 0x1.745d1745d1746p-4; // 1/11
  p = p * w + 0x1.c71c71c71c71cp-4; // 1/9
  p = p * w + 0x1.2492492492492p-3; // 1/7
  p = p * w + 0x1.999999999999ap-3; // 1/5
  p = p * w + 0x1.5555555555555p-2; // 1/3
  p = p * w + 1.0;
  return p;
}

// Natural logarithm for finite x > 0: x = 2^e * m with m in [sqrt(1/2),
// sqrt(2)], log(m) = 2 atanh((m-1)/(m+1)).
MMC_HD double log(double x) {
  if (!(x > 0.0)) return x == 0.0 ? -bitsd(0x7ff0000000000000ULL) : bitsd(0x7ff8000000000000ULL);
  uint64_t b = dbits(x);
  int e = (int)((b >> 52) & 0x7ff);
  if (e == 0x7ff) return x;  // +inf
  if (e == 0) {              // subnormal: scale into the normal range
    x = x * 0x1p54;
    b = dbits(x);
    e = (int)((b >> 52) & 0x7ff) - 54;
  }
  e -= 1023;
  double m = bitsd((b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);
  if (m > MMCM_SQRT2) {
    m = m * 0.5;
    e += 1;
  }
  double s = (m - 1.0) / (m + 1.0);
  double lnm = 2.0 * s * atanh_series(s * s);
  double de = (double)e;
  return de * MMCM_LN2_HI + (de * MMCM_LN2_LO + lnm);
}

// log(1+u) for u >= 0 without cancellation near 0.
MMC_HD double log1p_pos(double u) {
  if (u < 0.4) {
    double s = u / (2.0 + u);
    return 2.0 * s * atanh_series(s * s);
  }
  return mmcm::log(1.0 + u);
}

// Inverse hyperbolic sine via the identities
//   asinh(a) = log(2a) for large a, log(2a + 1/(sqrt(a^2+1)+a)) for a > 2,
//   log1p(a + a^2/(1+sqrt(1+a^2))) otherwise; odd symmetry for a < 0.
MMC_HD double asinh(double t) {
  double a = dabs(t);
  double r;
  if (a < 0x1p-28) {
    r = a;
  } else if (a > 0x1p28) {
    r = mmcm::log(a) + MMCM_LN2;
  } else if (a > 2.0) {
    r = mmcm::log(2.0 * a + 1.0 / (dsqrt(a * a + 1.0) + a));
  } else {
    double a2 = a * a;
    r = log1p_pos(a + a2 / (1.0 + dsqrt(1.0 + a2)));
  }
  return t < 0.0 ? -r : r;
}

// atan(x)/x = sum_k (-1)^k x^(2k)/(2k+1) for |x| <= 0.4375 (23 terms).
MMC_HD double atan_series(double w) {
  double p = 0x1.6c16c16c16c17p-6;   // +1/45
  p = p * w - 0x1.7d05f417d05f4p-6;  // -1/43
  p = p * w + 0x1.8f9c18f9c18fap-6;  // +1/41
  p = p * w - 0x1.a41a41a41a41ap-6;  // -1/39
  p = p * w + 0x1.bacf914c1bad0p-6;  // +1/37
  p = p * w - 0x1.d41d41d41d41dp-6;  // -1/35
  p = p * w + 0x1.f07c1f07c1f08p-6;  // +1/33
  p = p * w - 0x1.0842108421084p-5;  // -1/31
  p = p * w + 0x1.1a7b9611a7b96p-5;  // +1/29
  p = p * w - 0x1.2f684bda12f68p-5;  // -1/27
  p = p * w + 0x1.47ae147ae147bp-5;  // +1/25
  p = p * w - 0x1.642c8590b2164p-5;  // -1/23
  p = p * w + 0x1.8618618618618p-5;  // +1/21
  p = p * w - 0x1.af286bca1af28p-5;  // -1/19
  p = p * w + 0x1.e1e1e1e1e1e1ep-5;  // +1/17
  p = p * w - 0x1.1111111111111p-4;  // -1/15
  p = p * w + 0x1.3b13b13b13b14p-4;  // +1/13
  p = p * w - 0x1.745d1745d1746p-4;  // -1/11
  p = p * w + 0x1.c71c71c71c71cp-4;  // +1/9
  p = p * w - 0x1.2492492492492p-3;  // -1/7
  p = p * w + 0x1.999999999999ap-3;  // +1/5
  p = p * w - 0x1.5555555555555p-2;  // -1/3
  p = p * w + 1.0;
  return p;
}

// Arctangent.  The argument is reduced with atan(a) = atan(c) +
// atan((a-c)/(1+a c)) for c in {1/2, 1, 3/2} and atan(a) = pi/2 - atan(1/a),
// using breakpoints 7/16, 11/16, 19/16, 39/16, so that the series argument
// satisfies |x| <= 7/16.
MMC_HD double atan(double t) {
  double a = dabs(t);
  double x, hi, lo;
  if (a >= 2.4375) {
    x = -1.0 / a;
    hi = MMCM_PIO2_HI;
    lo = MMCM_PIO2_LO;
  } else if (a >= 1.1875) {
    x = (a - 1.5) / (1.0 + 1.5 * a);
    hi = MMCM_ATAN_3HALF_HI;
    lo = MMCM_ATAN_3HALF_LO;
  } else if (a >= 0.6875) {
    x = (a - 1.0) / (a + 1.0);
    hi = MMCM_PIO4_HI;
    lo = MMCM_PIO4_LO;
  } else if (a >= 0.4375) {
    x = (2.0 * a - 1.0) / (2.0 + a);
    hi = MMCM_ATAN_HALF_HI;
    lo = MMCM_ATAN_HALF_LO;
  } else {
    x = a;
    hi = 0.0;
    lo = 0.0;
  }
  double p = x * atan_series(x * x);
  double r = hi + (lo + p);
  return t < 0.0 ? -r : r;
}

// exp(x): x = k ln2 + r, |r| <= ln2/2, exp(r) by an 18-term Taylor sum,
// then scaled by 2^k.  Results below ~1e-323 flush to zero.
MMC_HD double exp(double x) {
  if (x < -745.0) return 0.0;
  if (x > 709.5) return bitsd(0x7ff0000000000000ULL);
  double kf = dfloor(x * MMCM_INV_LN2 + 0.5);
  double r = (x - kf * MMCM_LN2_HI) - kf * MMCM_LN2_LO;
  double p = 0x1.952c77030ad4ap-49;   // 1/17!
  p = p * r + 0x1.ae7f3e733b81fp-45;  // 1/16!
  p = p * r + 0x1.ae7f3e733b81fp-41;  // 1/15!
  p = p * r + 0x1.93974a8c07c9dp-37;  // 1/14!
  p = p * r + 0x1.6124613a86d09p-33;  // 1/13!
  p = p * r + 0x1.1eed8eff8d898p-29;  // 1/12!
  p = p * r + 0x1.ae64567f544e4p-26;  // 1/11!
  p = p * r + 0x1.27e4fb7789f5cp-22;  // 1/10!
  p = p * r + 0x1.71de3a556c734p-19;  // 1/9!
  p = p * r + 0x1.a01a01a01a01ap-16;  // 1/8!
  p = p * r + 0x1.a01a01a01a01ap-13;  // 1/7!
  p = p * r + 0x1.6c16c16c16c17p-10;  // 1/6!
  p = p * r + 0x1.1111111111111p-7;   // 1/5!
  p = p * r + 0x1.5555555555555p-5;   // 1/4!
  p = p * r + 0x1.5555555555555p-3;   // 1/3!
  p = p * r + 0.5;
  p = p * r + 1.0;
  p = p * r + 1.0;
  int k = (int)kf;
  if (k < -1000) {
    p = p * 0x1p-64;
    k += 64;
  }
  return p * bitsd((uint64_t)(k + 1023) << 52);
}

// sin(pi t) and cos(pi t): t = n/2 + r with |r| <= 1/4, then Taylor sums in
// y = pi r (|y| <= pi/4) and a quadrant swap.
MMC_HD void sincospi(double t, double* sp, double* cp) {
  double n2 = dfloor(2.0 * t + 0.5);
  double r = t - 0.5 * n2;
  double q4 = n2 - 4.0 * dfloor(n2 * 0.25);
  int q = (int)q4;
  double y = r * MMCM_PI_HI + r * MMCM_PI_LO;
  double w = y * y;
  double s = 0x1.71b8ef6dcf572p-66;    // +1/21!
  s = s * w - 0x1.2f49b46814157p-57;   // -1/19!
  s = s * w + 0x1.952c77030ad4ap-49;   // +1/17!
  s = s * w - 0x1.ae7f3e733b81fp-41;   // -1/15!
  s = s * w + 0x1.6124613a86d09p-33;   // +1/13!
  s = s * w - 0x1.ae64567f544e4p-26;   // -1/11!
  s = s * w + 0x1.71de3a556c734p-19;   // +1/9!
  s = s * w - 0x1.a01a01a01a01ap-13;   // -1/7!
  s = s * w + 0x1.1111111111111p-7;    // +1/5!
  s = s * w - 0x1.5555555555555p-3;    // -1/3!
  s = s * w + 1.0;
  s = s * y;
  double c = 0x1.e542ba4020225p-62;    // +1/20!
  c = c * w - 0x1.6827863b97d97p-53;   // -1/18!
  c = c * w + 0x1.ae7f3e733b81fp-45;   // +1/16!
  c = c * w - 0x1.93974a8c07c9dp-37;   // -1/14!
  c = c * w + 0x1.1eed8eff8d898p-29;   // +1/12!
  c = c * w - 0x1.27e4fb7789f5cp-22;   // -1/10!
  c = c * w + 0x1.a01a01a01a01ap-16;   // +1/8!
  c = c * w - 0x1.6c16c16c16c17p-10;   // -1/6!
  c = c * w + 0x1.5555555555555p-5;    // +1/4!
  c = c * w - 0.5;                     // -1/2!
  c = c * w + 1.0;
  switch (q) {
    case 0: *sp = s; *cp = c; break;
    case 1: *sp = c; *cp = -s; break;
    case 2: *sp = -s; *cp = -c; break;
    default: *sp = -c; *cp = s; break;
  }
}

// ------------------------------------------------------------------ Philox
struct u32x4 {
  uint32_t x, y, z, w;
};

#if defined(__CUDACC__)
// The multipliers in the constant bank on the device: a wide multiply takes a
// constant-bank operand directly, where a literal would first be moved into a
// register before each multiply (the sweep kernels have none to keep it in).
static __constant__ uint32_t philox_mul_dev[2] = {0xD2511F53u, 0xCD9E8D57u};
#endif

MMC_HD u32x4 philox_round(u32x4 c, uint32_t k0, uint32_t k1) {
#if defined(__CUDA_ARCH__)
  const uint32_t M0 = philox_mul_dev[0], M1 = philox_mul_dev[1];
#else
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
#endif
  // one 32 x 32 -> 64-bit product per multiplier (a single wide multiply-add
  // on the GPU); hi and lo are its halves
  const uint64_t p0 = (uint64_t)M0 * c.x, p1 = (uint64_t)M1 * c.z;
  const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
  const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
  u32x4 r;
  r.x = hi1 ^ c.y ^ k0;
  r.y = lo1;
  r.z = hi0 ^ c.w ^ k1;
  r.w = lo0;
  return r;
}

// Ten rounds, key bumped by the Weyl constants between rounds.
MMC_HD u32x4 philox4x32_10(u32x4 c, uint32_t k0, uint32_t k1) {
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int i = 0; i < 9; ++i) {
    c = philox_round(c, k0, k1);
    k0 += W0;
    k1 += W1;
  }
  return philox_round(c, k0, k1);
}

// Stream tags for the fourth counter word.
enum : uint32_t { STREAM_SWEEP = 0u, STREAM_INIT = 1u, STREAM_SWAP = 2u };

// Uniform in (0,1): (r + 1/2) 2^-32, exact in FP64.
MMC_HD double u01_f64(uint32_t r) { return ((double)r + 0.5) * 0x1p-32; }
// Uniform in (0,1) with 23 random bits, exact in FP32.
MMC_HD float u01_f32(uint32_t r) { return ((float)(r >> 9) + 0.5f) * 0x1p-23f; }

}  // namespace mmcm
