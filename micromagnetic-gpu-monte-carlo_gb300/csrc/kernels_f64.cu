// kernels_f64.cu -- FP64 instantiation of the hot-path kernels, the FP64
// transform of the demag tensor and small utility kernels.  Built with
// -fmad=false: the FP64 sweep, its proposals and exp() then round exactly like
// the CPU oracle built with -ffp-contract=off.
#include <curand_kernel.h>

#include <atomic>

#include "coef.h"
#include "fused2d.cuh"
#include "grad.cuh"
#include "kernels.cuh"

namespace mmc {
MMC_INSTANTIATE_LAUNCHERS(double)
static_assert(MCT == MC_TILE_SIDE, "tile side");
bool mc_tile_eligible(const Geom& g) { return mc_tile_ok(g); }
bool mc_quad_eligible(const Geom& g) { return mc_quad_ok(g); }
bool mc_band_eligible(const Geom& g) { return mc_band_ok(g); }
bool mc_strip_eligible(const Geom& g) { return mc_strip_ok(g); }
size_t mc_strip_smem_bytes(const Geom& g, size_t real_size) {
  return real_size == 4 ? mc_strip_smem<float>(g) : mc_strip_smem<double>(g);
}
bool mc_pipe_eligible(const Geom& g) { return mc_pipe_ok(g); }
size_t mc_pipe_smem_bytes(const Geom& g, size_t real_size) {
  return real_size == 4 ? mc_pipe_smem<float>(g) : mc_pipe_smem<double>(g);
}
MMC_INSTANTIATE_FUSED(double)
MMC_INSTANTIATE_GRAD(double)

int energy_partials_count(const Geom& g) { return energy_blocks(g); }

size_t grid_barrier_bytes() { return sizeof(GridBarrier); }
int grid_barrier_error(const GridBarrier* b) { return b->err; }

// Failure-detection self-test: one CTA waits at a grid barrier for one more
// arrival than the grid has, so the wait can only end by its poll budget; the
// kernel records the timeout in the barrier's error word and returns.
static __global__ void k_barrier_timeout_selftest(GridBarrier* bar, unsigned long long spin_limit, int* ok_out) {
  __shared__ int flag;
  unsigned int target = 0;
  const bool ok = grid_sync(bar, target, &flag, spin_limit, gridDim.x + 1);
  if (threadIdx.x == 0) *ok_out = ok ? 1 : 0;
}

cudaError_t launch_barrier_timeout_selftest(void* bar, unsigned long long spin_limit, int* ok_out) {
  k_barrier_timeout_selftest<<<1, 32>>>(reinterpret_cast<GridBarrier*>(bar), spin_limit, ok_out);
  return cudaGetLastError();
}

// Failure-detection self-test of k_mc_pipe's bounded buffer wait: an mbarrier
// that expects one arrival that never comes (and no copy), so the wait can
// only end by its time limit.
static __global__ void k_mbar_timeout_selftest(unsigned long long limit_ns, int* timed_out) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *timed_out = mbar_wait_bounded(&bar, 0u, limit_ns) ? 0 : 1;
  }
}

cudaError_t launch_mbar_timeout_selftest(unsigned long long limit_ns, int* timed_out) {
  k_mbar_timeout_selftest<<<1, 32>>>(limit_ns, timed_out);
  return cudaGetLastError();
}

// k_mc_pipe's error word (one per device): set by a CTA whose buffer wait ran
// out of its time limit.
__device__ int g_mc_pipe_err;

int* mc_pipe_err_word() {
  static std::atomic<int*> words[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  int* p = words[dev].load();
  if (!p) {
    void* a = nullptr;
    if (cudaGetSymbolAddress(&a, g_mc_pipe_err) != cudaSuccess) return nullptr;
    p = static_cast<int*>(a);
    words[dev].store(p);
  }
  return p;
}

int mc_pipe_error_take() {
  int* p = mc_pipe_err_word();
  int v = 0;
  if (!p || cudaMemcpy(&v, p, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return 0;
  if (v) cudaMemset(p, 0, sizeof(int));
  return v;
}

// Forward transform of the six real tensor blocks k6[c][z][y][x] (padded
// grid) into spec64[c][kz][ky][kx] (src/main.cu:593-642 ran cuFFT D2Z here).
cudaError_t launch_tensor_fft(const Geom& g, const FftPlan& px, const FftPlan& py, const FftPlan& pz,
                              const DemagTuning& tun, const double* k6, double2* spec64, cudaStream_t st) {
  const long long ns = g.nspec;
  MMC_TRY(cudaMemsetAsync(spec64, 0, 6 * (size_t)ns * sizeof(double2), st));
  MMC_TRY(run_x_forward<double>(px, 6, g.nxp, g.nyp, g.nyp * g.nzp, k6, g.np, spec64, ns, g.nyp, g.hx, g.hxp, 1,
                                tun.x_threads, st, 1, 0, 0));
  const long long ystride = g.hxp, yplane = (long long)g.nyp * g.hxp;
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

__global__ void k_advance(SweepCounters* ctr, uint32_t delta, int count) {
  pdl_wait();  // the previous kernels read the counters
  if ((int)threadIdx.x < count) ctr[threadIdx.x].sweep += delta;
}

cudaError_t launch_advance(SweepCounters* ctr, uint32_t delta, cudaStream_t st, int count) {
  if (count < 1 || count > 32) return cudaErrorInvalidValue;
  return launch_pdl(k_advance, dim3(1), dim3(32), 0, st, ctr, delta, count);
}

// One parallel-tempering pass: in each ladder, the temperature pairs (k, k+1)
// with k = round mod 2, 2 + round mod 2, ... attempt a swap with probability
// min(1, exp((1/kT_k - 1/kT_k+1)(E_k - E_k+1))), E from the energy kernel's
// per-replica sums; u = Philox(key; ladder, round, k, STREAM_SWAP).  A swap
// exchanges the two replicas' temperatures and recomputes their coefficients.
template <typename T>
__global__ void k_pt_swap(PtDevice pt, const McParams* __restrict__ params, McCoef<T>* __restrict__ coef,
                          const double* __restrict__ red) {
  const unsigned int round = *pt.round;
  for (int l = threadIdx.x; l < pt.nladders; l += blockDim.x) {
    const double kB = 1.3806488e-23;
    unsigned long long att = 0, acc = 0;
    for (int k = (int)(round & 1u); k + 1 < pt.K; k += 2) {
      const int ra = pt.replica_at[l * pt.K + k], rb = pt.replica_at[l * pt.K + k + 1];
      const double* qa = red + (size_t)ra * NQ;
      const double* qb = red + (size_t)rb * NQ;
      const double Ea = qa[0] + qa[1] + qa[2] + qa[3] + qa[4];
      const double Eb = qb[0] + qb[1] + qb[2] + qb[3] + qb[4];
      const double Ta = pt.temps[l * pt.K + k], Tb = pt.temps[l * pt.K + k + 1];
      const double delta = (1.0 / (kB * Ta) - 1.0 / (kB * Tb)) * (Ea - Eb);
      mmcm::u32x4 ctr = {(uint32_t)l, round, (uint32_t)k, mmcm::STREAM_SWAP};
      const double u = mmcm::u01_f64(mmcm::philox4x32_10(ctr, pt.key0, pt.key1).x);
      ++att;
      if (delta >= 0.0 || u < mmcm::exp(delta)) {
        ++acc;
        pt.replica_at[l * pt.K + k] = rb;
        pt.replica_at[l * pt.K + k + 1] = ra;
        pt.replica_T[ra] = Tb;
        pt.replica_T[rb] = Ta;
        coef[ra] = mc_coef_from<T>(params[ra], Tb);
        coef[rb] = mc_coef_from<T>(params[rb], Ta);
      }
    }
    atomicAdd(&pt.counts[0], att);
    atomicAdd(&pt.counts[1], acc);
  }
  __syncthreads();
  if (threadIdx.x == 0) *pt.round = round + 1u;
}

template <typename T>
cudaError_t launch_pt_swap(const PtDevice& pt, const McParams* params, McCoef<T>* coef, const double* red,
                           cudaStream_t st) {
  k_pt_swap<T><<<1, 64, 0, st>>>(pt, params, coef, red);
  return cudaGetLastError();
}
template cudaError_t launch_pt_swap<float>(const PtDevice&, const McParams*, McCoef<float>*, const double*,
                                           cudaStream_t);
template cudaError_t launch_pt_swap<double>(const PtDevice&, const McParams*, McCoef<double>*, const double*,
                                            cudaStream_t);

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
