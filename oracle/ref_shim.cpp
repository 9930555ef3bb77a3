// ref_shim.cpp -- C entry points around the reference's own demag code.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_ref.py compiles this file with g++
// against the reference's unmodified src/demag_cu.cu (included below, read in
// place from the reference checkout) and the stand-in headers of
// oracle/ref_stubs/, producing oracle/_ref/libref_demag.so (FLOAT2 = float2,
// the reference's default) and oracle/_ref/libref_demag_f64.so (built with
// USE_DOULBE_IN_GPU, FLOAT2 = double2, src/constant.h:41-51).  Nothing in the
// product loads these libraries; tests/golden/make_ref_golden.py and the CPU
// tests use them to pin the oracle to the reference's arithmetic.
//
// What runs is the reference's code, not a restatement:
//  - ref_f_host / ref_g_host: ktensorcpu::f, ktensorcpu::g (src/demag_cu.h:43-71);
//  - ref_f_devsrc / ref_g_devsrc: the GPU-side f, g (src/demag_cu.cu:16-44)
//    compiled for the host;
//  - ref_ktensor: ktensorcpu::ktensorCPU (src/demag_cu.cu:119-248), whose
//    trailing "device" copies land in the caller's host arrays;
//  - ref_hexchange: calHexchangeKernel (src/demag_cu.cu:68-116), every thread
//    of the reference's launch grid (dimBlock 5x5x1 and dimGrid over the padded
//    dims, src/main.cu:272-281, launch :876-880) run in turn on the host.
#include "demag_cu.cu"

#include <cstdint>

extern "C" {

double ref_f_host(double x, double y, double z) { return ktensorcpu::f(x, y, z); }
double ref_g_host(double x, double y, double z) { return ktensorcpu::g(x, y, z); }
double ref_f_devsrc(double x, double y, double z) { return ::f(x, y, z); }
double ref_g_devsrc(double x, double y, double z) { return ::g(x, y, z); }

// Bytes of one FLOAT2 in this build: 8 (float2) or 16 (double2).
int ref_float2_bytes(void) { return (int)sizeof(FLOAT2); }

// The reference's CONST_PI (src/constant.h:21).
double ref_const_pi(void) { return CONST_PI; }

// Tensor of the padded grid in the reference's layout: six blocks (xx, xy, xz,
// yy, yz, zz) of nxp*nyp*nzp doubles, index z + nzp*(y + nyp*x) (z fastest,
// src/demag_cu.cu:146).  pbc_* are image counts (>= 0).  Returns the number of
// tensor points ktensorCPU visited.
long ref_ktensor(int nxp, int nyp, int nzp, double dx, double dy, double dz, int pbc_x, int pbc_y,
                 int pbc_z, double* k6) {
  const long np = (long)nxp * nyp * nzp;
  bool quit = false;
  ktensorcpu::ktensorCPU(nxp, nyp, nzp, dx, dy, dz, pbc_x, pbc_y, pbc_z, k6, k6 + np, k6 + 2 * np,
                         k6 + 3 * np, k6 + 4 * np, k6 + 5 * np, quit);
  return np;
}

// H^ = K^ . M^ / N over the padded grid (complex arrays of nxp*nyp*nzp FLOAT2,
// the reference's index z + nzp*(y + nyp*x)).  m3: the three spectra back to
// back; k6: the six tensor spectra (xx, xy, xz, yy, yz, zz); h3: output.
void ref_hexchange(int nxp, int nyp, int nzp, const void* m3, const void* k6, void* h3) {
  const long np = (long)nxp * nyp * nzp;
  FLOAT2* M = (FLOAT2*)m3;
  FLOAT2* K = (FLOAT2*)k6;
  FLOAT2* H = (FLOAT2*)h3;
  blockDim = dim3{5u, 5u, 1u};
  gridDim = dim3{(unsigned)((nxp + 4) / 5), (unsigned)((nyp + 4) / 5), (unsigned)nzp};
  for (unsigned bz = 0; bz < gridDim.z; ++bz)
    for (unsigned by = 0; by < gridDim.y; ++by)
      for (unsigned bx = 0; bx < gridDim.x; ++bx)
        for (unsigned tz = 0; tz < blockDim.z; ++tz)
          for (unsigned ty = 0; ty < blockDim.y; ++ty)
            for (unsigned tx = 0; tx < blockDim.x; ++tx) {
              blockIdx = uint3{bx, by, bz};
              threadIdx = uint3{tx, ty, tz};
              calHexchangeKernel(nxp, nyp, nzp, M, M + np, M + 2 * np, K, K + np, K + 2 * np, K + 3 * np,
                                 K + 4 * np, K + 5 * np, H, H + np, H + 2 * np);
            }
}

}  // extern "C"
