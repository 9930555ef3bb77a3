// kernels_f64.cu -- FP64 instantiation of the hot-path kernels, the FP64
// transform of the demag tensor and small utility kernels.  Built with
// -fmad=false: the FP64 sweep, its proposals and exp() then round exactly like
// the CPU oracle built with -ffp-contract=off.
#include <curand_kernel.h>

#include "fused2d.cuh"
#include "kernels.cuh"

namespace mmc {
MMC_INSTANTIATE_LAUNCHERS(double)
MMC_INSTANTIATE_FUSED(double)

int energy_partials_count(const Geom& g) { return energy_blocks(g); }

size_t grid_barrier_bytes() { return sizeof(GridBarrier); }
int grid_barrier_error(const GridBarrier* b) { return b->err; }

// Forward transform of the six real tensor blocks k6[c][z][y][x] (padded
// grid) into spec64[c][kz][ky][kx] (src/main.cu:593-642 ran cuFFT D2Z here).
cudaError_t launch_tensor_fft(const Geom& g, const FftPlan& px, const FftPlan& py, const FftPlan& pz,
                              const DemagTuning& tun, const double* k6, double2* spec64, cudaStream_t st) {
  const long long ns = g.nspec;
  MMC_TRY(run_x_forward<double>(px, 6, g.nxp, g.nyp, g.nyp * g.nzp, k6, g.np, spec64, ns, g.nyp, g.hx, 1,
                                tun.x_threads, st));
  const long long ystride = g.hx, yplane = (long long)g.nyp * g.hx;
  for (int half = 0; half < 2; ++half) {
    double2* S = spec64 + 3 * half * ns;
    if (g.nyp > 1)
      MMC_TRY(run_col_pass<double>(py, 3, S, ns, nullptr, g.hx, g.nzp, yplane, ystride, g.nyp, g.nyp, PASS_FWD, 1.0,
                                   tun.col_tx, tun.col_threads, st));
    if (g.nzp > 1)
      MMC_TRY(run_col_pass<double>(pz, 3, S, ns, nullptr, g.hx, g.nyp, ystride, yplane, g.nzp, g.nzp, PASS_FWD, 1.0,
                                   tun.col_tx, tun.col_threads, st));
  }
  return cudaSuccess;
}

__global__ void k_advance(SweepCounters* ctr, uint32_t delta) { ctr->sweep += delta; }

cudaError_t launch_advance(SweepCounters* ctr, uint32_t delta, cudaStream_t st) {
  k_advance<<<1, 1, 0, st>>>(ctr, delta);
  return cudaGetLastError();
}

// Philox cross-check against cuRAND's device implementation (test hook).
__global__ void k_philox_selftest(long long n, const uint32_t* __restrict__ ctr, uint32_t k0, uint32_t k1,
                                  uint32_t* __restrict__ out, uint32_t* __restrict__ out_curand) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  mmcm::u32x4 c = {ctr[4 * i], ctr[4 * i + 1], ctr[4 * i + 2], ctr[4 * i + 3]};
  mmcm::u32x4 r = mmcm::philox4x32_10(c, k0, k1);
  out[4 * i] = r.x;
  out[4 * i + 1] = r.y;
  out[4 * i + 2] = r.z;
  out[4 * i + 3] = r.w;
  uint4 cc = make_uint4(c.x, c.y, c.z, c.w);
  uint4 rc = curand_Philox4x32_10(cc, make_uint2(k0, k1));
  out_curand[4 * i] = rc.x;
  out_curand[4 * i + 1] = rc.y;
  out_curand[4 * i + 2] = rc.z;
  out_curand[4 * i + 3] = rc.w;
}

cudaError_t launch_philox_selftest(long long n, const uint32_t* ctr, uint32_t k0, uint32_t k1, uint32_t* out,
                                   uint32_t* out_curand, cudaStream_t st) {
  k_philox_selftest<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(n, ctr, k0, k1, out, out_curand);
  return cudaGetLastError();
}

}  // namespace mmc
