// mmc_internal.h -- structures shared by the host runtime and the kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mmc {

// Division by a run-time invariant d >= 1 as a multiply-high, an add and a
// shift (Granlund & Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994): with l = ceil(log2 d) and
// m = floor(2^32 (2^l - d) / d) + 1, n / d = (umulhi(m, n) + n) >> l for
// 0 <= n < 2^31.  The kernels' index arithmetic divides by lattice and
// transform sizes that are only known at run time.
#ifdef __CUDACC__
#define MMC_HDI __host__ __device__
#else
#define MMC_HDI
#endif
struct FastDiv {
  uint32_t d = 1, m = 1, l = 0;
  FastDiv() = default;
  MMC_HDI explicit FastDiv(uint32_t dd) : d(dd ? dd : 1) {
    l = 0;
    while ((1ull << l) < d) ++l;
    m = (uint32_t)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
  }
#ifdef __CUDACC__
  __device__ __forceinline__ int div(int n) const { return (int)((__umulhi(m, (uint32_t)n) + (uint32_t)n) >> l); }
  __device__ __forceinline__ int mod(int n) const { return n - div(n) * (int)d; }
#endif
};

constexpr int FFT_MAX_STAGES = 24;
constexpr int FFT_MAX_RADIX = 31;  // largest prime factor an FFT length may have

// Mixed-radix Stockham plan for one transform length.  Stage s has radix
// radix[s] and ns[s] = product of the earlier radices.  Twiddles of stage s
// live at tw_off[s]: entry (t-1)*ns + k = exp(-2 pi i t k / (ns*radix)) for
// t in [1, radix), k in [0, ns); the radix-th roots of unity exp(-2 pi i m /
// radix) live at root_off[s].
struct FftPlan {
  int n;
  int nstages;
  int radix[FFT_MAX_STAGES];
  int ns[FFT_MAX_STAGES];
  int tw_off[FFT_MAX_STAGES];
  int root_off[FFT_MAX_STAGES];
  int tw_total;
  // Warp-level transform for power-of-two lengths n = A * B (A values per lane,
  // B lanes per line): warp_a = A (0 = use the Stockham stages), and the n
  // roots exp(-2 pi i j / n) at full_off.
  int warp_a, warp_b;
  int full_off;
  FastDiv dn;  // n
  FastDiv dnb[FFT_MAX_STAGES];  // n / radix[s]
  FastDiv dns[FFT_MAX_STAGES];  // ns[s]
  const double2* tw64;
  const float2* tw32;
};

// Lattice geometry.  Cell i = x + nx*(y + ny*z).  The tensor grid (txp, typ,
// tzp) follows src/main.cu:254-263 of the reference (open axis n -> 2n - 1,
// periodic n); the transform grid (nxp, nyp, nzp) equals it except that an
// open axis of 2n - 1 > 16 is padded further to the next power of two up to
// 1024, where the warp-level transforms apply.  The spectrum keeps the
// kx half-axis: hx = nxp/2 + 1 columns stored with an even row pitch hxp (so
// that pairs of FP32 columns are 16-byte aligned), layout [comp][kz][ky][kx],
// nspec = hxp*nyp*nzp.  Pad columns hold zeros.
struct Geom {
  int nx, ny, nz;
  int nxp, nyp, nzp;  // the transform grid (the tensor grid, open axes possibly padded further)
  int txp, typ, tzp;  // the tensor grid: the reference's padded dims
  int hx;
  int hxp;
  int per[3];      // periodic neighbours on this axis (pbc != 0)
  int ncolors;     // 2, or 3 when a periodic axis has odd length
  long long n;     // nx*ny*nz
  long long np;    // nxp*nyp*nzp
  long long tnp;   // txp*typ*tzp
  long long nspec; // hxp*nyp*nzp
  FastDiv dnx, dny, dhx, dhxc;  // nx, ny, hx, (nx + 1) / 2
};

// Metropolis coefficients, all in units of kT (see the sweep kernel).  16-byte
// aligned: a sweep thread copies its replica's set with 16-byte loads.
template <typename T>
struct alignas(16) McCoef {
  T wex[3];   // 2 Aex V / (d_a^2 kT)
  T wdm[2];   // Dind V / (d_a kT), a = x, y
  T can;      // Ku1 V / kT
  T u[3];     // anisotropy axis (unit)
  T cz[3];    // Ms V B / kT
  T cd;       // mu0 Ms^2 V / kT, 0 when demag is off
  T k0[6];    // self tensor xx, xy, xz, yy, yz, zz
  T k0h[6];   // cd / 2 * k0 (the FP32 form of dE)
  uint32_t key0, key1;  // Philox key = seed
};

// Energy prefactors (SI, J).
struct EnCoef {
  double aexV_d2[3];  // Aex V / d_a^2
  double dV_2d[2];    // Dind V / (2 d_a)
  double kuV;         // Ku1 V
  double u[3];
  double msVB[3];     // Ms V B
  double demag;       // mu0 Ms^2 V / 2, 0 when demag is off
};

// Effective-field prefactors (A/m).
struct HCoef {
  double ex_d2[3];  // 2 Aex / (mu0 Ms d_a^2)
  double dm_2d[2];  // 2 Dind / (mu0 Ms) / (2 d_a)
  double an;        // 2 Ku1 / (mu0 Ms)
  double u[3];
  double b[3];      // B / mu0
  double ms;        // Ms, 0 when demag is off
};

// Number of reduced quantities produced by the energy kernel:
// E_ex, E_dmi, E_an, E_zeeman, E_demag, sum mx, sum my, sum mz, sum solid angle.
constexpr int NQ = 9;

// Shared-memory line stride (elements) of the column passes for a transform
// plan and complex size csize: room for the padded transpose rows of the
// warp-level transforms (n + warp_a - 1 elements), plus a padding that spreads
// the tile's 8 columns over the banks (+2 for 8-byte FP32 complex values,
// whose 16-lane wavefronts then touch distinct banks; +1 for 16-byte FP64
// ones).
MMC_HDI inline int col_line_stride(const FftPlan& p, size_t csize) {
  return p.n + p.warp_a + (csize == 8 ? 2 : 1);
}

// Launch shapes chosen by the host (autotuned).
struct DemagTuning {
  int x_rows_per_cta;
  int x_threads;
  int col_tx;      // kx columns per tile in the y pass
  int col_tx_z;    // kx columns per tile in the z pass
  int col_threads;
  int mc_form;     // MC_FORM_*
  int fft_inline;  // 1: the pass kernels expand the warp-level transforms in line
  int col_lean;    // 1: column passes transform in place and read K^ from global memory; 2: as 1, and
                   // film y passes of length 64 or 256 hold their lines in registers (k_col_reg); 3: as 2,
                   // one component per thread (k_col_reg3)
};

// Device counters read by the sweep kernels: [stage, sweep].
struct SweepCounters {
  uint32_t stage;
  uint32_t sweep;
};

// ------------------------------------------------------------- launchers
// Implemented in kernels_f32.cu / kernels_f64.cu (T = float / double) and newell.cu.
// Batched forms: nrep replicas of one geometry stored back to back (m and h
// with stride 3n, the spectrum with stride 3 nspec, one McCoef / EnCoef and
// one accept counter per replica); the tensor spectrum is shared.
template <typename T>
cudaError_t launch_demag(const Geom& g, const FftPlan& px, const FftPlan& py, const FftPlan& pz,
                         const DemagTuning& tun, const T* m, T* h, void* spec, const void* khat,
                         cudaStream_t st, int nrep = 1, cudaEvent_t* ev = nullptr);
// Metropolis kernel forms (all make the same decisions): one scalar launch
// per colour; both colours of a film in one tile launch; one vectorised launch
// per colour for films with nx a multiple of 4.
// (MC_FORM_BAND: the vectorised form with the CTA's rows staged in shared
// memory by asynchronous copies.)  MC_FORM_STRIP: both colours of a film in
// one launch by strips of rows, reading m from one buffer and writing the
// other (launch_mc_strip; the batch alternates its two copies of m).
// MC_FORM_PIPE: one colour per launch by persistent CTAs, each band's rows
// staged by bulk asynchronous copies into a ring of shared-memory buffers
// (k_mc_pipe).
enum : int {
  MC_FORM_SCALAR = 0,
  MC_FORM_TILE = 1,
  MC_FORM_QUAD = 2,
  MC_FORM_BAND = 3,
  MC_FORM_STRIP = 4,
  MC_FORM_PIPE = 5
};
// color < 0: every colour of the sweep in the given form (falls back to the
// scalar form where the lattice does not qualify).
template <typename T>
cudaError_t launch_mc(const Geom& g, const McCoef<T>* c, T* m, const T* h, const SweepCounters* ctr,
                      int color, unsigned long long* acc, cudaStream_t st, int nrep = 1, int form = 0);
// Whether a lattice can use the tile form (and its tile side) or the vector form.
bool mc_tile_eligible(const Geom& g);
bool mc_quad_eligible(const Geom& g);
bool mc_band_eligible(const Geom& g);
bool mc_strip_eligible(const Geom& g);
size_t mc_strip_smem_bytes(const Geom& g, size_t real_size);
bool mc_pipe_eligible(const Geom& g);
size_t mc_pipe_smem_bytes(const Geom& g, size_t real_size);
// k_mc_pipe's device error word on the current device (its address, cached),
// and its value, cleared when set (synchronous).
int* mc_pipe_err_word();
int mc_pipe_error_take();
// One sweep (both colours) in the strip form: m_in -> m_out (distinct buffers).
template <typename T>
cudaError_t launch_mc_strip(const Geom& g, const McCoef<T>* c, const T* m_in, T* m_out, const T* h,
                            const SweepCounters* ctr, unsigned long long* acc, cudaStream_t st, int nrep);
constexpr int MC_TILE_SIDE = 32;
template <typename T>
// with_q: 1 energies, <m> and Q; 0 energies and <m> (FP64 per cell); -1 the
// energies for tempering swaps (FP32 per cell, FP64 sums, for FP32 replicas;
// as 0 for FP64 ones).
cudaError_t launch_energy(const Geom& g, const EnCoef* e, const T* m, const T* h, double* partials,
                          int npartials, double* out, cudaStream_t st, int nrep = 1, int with_q = 1);
template <typename T>
cudaError_t launch_field(const Geom& g, const HCoef& c, int term, const T* m, const T* h, double* out,
                         cudaStream_t st);
template <typename T>
cudaError_t launch_init(const Geom& g, uint64_t seed, T* m, cudaStream_t st);
// Gradient and relaxation (grad.cuh).  launch_demag_sym convolves with the
// symmetrised tensor (spectrum Re K^).  launch_grad writes dE/dm (3n doubles,
// may be null) and 9 sums to out (see k_grad); launch_relax_eval writes
// [s.s, s.y, y.y, max torque] to out.
template <typename T>
cudaError_t launch_demag_sym(const Geom& g, const FftPlan& px, const FftPlan& py, const FftPlan& pz,
                             const DemagTuning& tun, const T* m, T* h, void* spec, const void* khat, cudaStream_t st);
template <typename T>
cudaError_t launch_grad(const Geom& g, const HCoef& c, const EnCoef& eu, double gscale, const T* m, const T* hs,
                        double* grad, double* partials, int npartials, double* out, cudaStream_t st);
template <typename T>
cudaError_t launch_relax_eval(const Geom& g, const HCoef& c, double inv_ms, const T* m, const T* hs, double* P,
                              const double* s, bool first, double* partials, int npartials, double* out,
                              cudaStream_t st);
template <typename T>
cudaError_t launch_relax_update(const Geom& g, T* m, const double* P, double tau, double* s, cudaStream_t st);
// Raises the dynamic shared-memory limit of every pass kernel (once per device).
template <typename T>
cudaError_t launch_prepare(int max_dyn_smem);
template <typename T>
cudaError_t launch_from_f64(long long count, const double* src, T* dst, cudaStream_t st);
template <typename T>
cudaError_t launch_to_f64(long long count, const T* src, double* dst, cudaStream_t st);
template <typename T>
cudaError_t launch_khat_store(long long count, const double2* spec64, void* khat, cudaStream_t st);

// FP64 setup: the Newell tensor (newell.cu) and its forward transform.
// far_r2 > 0: image offsets with squared distance >= far_r2 (m^2) use the
// far-field expansion (newell_far.h).  nodes: each image's sum as the 27-point
// stencil of node values (tensor_sum = 1) instead of its 64 terms.
cudaError_t launch_newell(const Geom& g, double dx, double dy, double dz, int Px, int Py, int Pz,
                          double pi, double* k6, int px0, int px1, int finalize, cudaStream_t st,
                          double far_r2 = 0.0, int nodes = 0);
// The tensor on the tensor grid -> the transform grid: offsets |o| <= n - 1
// copied, the offsets an open axis gains by the extra padding set to 0 (the
// convolution of n cells never reaches them).
cudaError_t launch_tensor_rewrap(const Geom& g, const double* k6t, double* k6f, cudaStream_t st);
cudaError_t launch_tensor_fft(const Geom& g, const FftPlan& px, const FftPlan& py, const FftPlan& pz,
                              const DemagTuning& tun, const double* k6, double2* spec64, cudaStream_t st);
// Advances the sweep counter of `count` (<= 32) consecutive SweepCounters.
cudaError_t launch_advance(SweepCounters* ctr, uint32_t delta, cudaStream_t st, int count = 1);
cudaError_t launch_philox_selftest(long long n, const uint32_t* ctr, uint32_t k0, uint32_t k1, uint32_t* out,
                                   uint32_t* out_curand, cudaStream_t st);

int energy_partials_count(const Geom& g);

// Persistent film engine (fused2d.cuh).
struct GridBarrier;
template <typename T>
struct FusedArgs {
  const McCoef<T>* coef;
  T* m;
  T* m2;  // second copy of m: the result of an odd sweep count lands here
  T* h;
  void* spec;
  void* spec2;
  const void* khat;
  unsigned long long* acc;
  GridBarrier* bar;
  unsigned long long* tbuf;  // optional phase timestamps, see fused2d.cuh
  uint32_t stage, sweep0;
  int nsweeps;
  int band;
};
constexpr int FUSED_STAMP_WORDS = 16 * 9 * 2;  // sweeps x points x (first CTA, last CTA)
template <typename T>
size_t fused2d_smem_bytes(const Geom& g, const FftPlan& px, const FftPlan& py, int band);
template <typename T>
cudaError_t fused2d_blocks_per_sm(const Geom& g, const FftPlan& px, const FftPlan& py, int band, int* out);
template <typename T>
cudaError_t launch_fused2d(const Geom& g, const FftPlan& px, const FftPlan& py, const FusedArgs<T>& a, int nblocks,
                           cudaStream_t st);
size_t grid_barrier_bytes();
// Address of the static spectrum array of mmc_demag_apply_static() on
// `device` (the current device); looked up on the first call per device.
cudaError_t demag_static_scratch(int device, void** out);

// Batched film sweeps (fused2d.cuh / rows.cuh): the row kernel (inverse x
// transform, both colours, forward x transform) and the 2-D column pass.
template <typename T>
size_t rows_smem_bytes(const Geom& g, const FftPlan& px, int band);
template <typename T>
cudaError_t rows_prepare(const Geom& g, const FftPlan& px, int band, int* blocks_per_sm);
template <typename T>
cudaError_t launch_rows(const Geom& g, const FftPlan& px, const McCoef<T>* coef, const T* m, T* mo, T* h,
                        const void* spec, void* spec_out, unsigned long long* acc, const SweepCounters* ctr, int band,
                        int nrep, bool with_h, bool do_forward, cudaStream_t st);
template <typename T>
cudaError_t launch_col_pass_2d(const Geom& g, const FftPlan& py, const DemagTuning& tun, void* spec,
                               const void* khat, cudaStream_t st, int nrep);

// Parallel tempering across the replicas of a batch (kernels_f64.cu).
// replica_at[l * K + k] is the replica holding temperature temps[l * K + k] of
// ladder l; round advances once per swap pass.
struct PtDevice {
  int nladders, K;
  int* replica_at;
  const double* temps;
  double* replica_T;
  unsigned int* round;
  unsigned long long* counts;  // [0] attempted, [1] accepted
  uint32_t key0, key1;
};
struct McParams;
template <typename T>
cudaError_t launch_pt_swap(const PtDevice& pt, const McParams* params, McCoef<T>* coef, const double* red,
                           cudaStream_t st);
int grid_barrier_error(const GridBarrier* host_copy);
// Test hook: a barrier wait that can only run out (see mmc_selftest_barrier_timeout).
cudaError_t launch_barrier_timeout_selftest(void* bar, unsigned long long spin_limit, int* ok_out);
// Test hook: k_mc_pipe's bounded buffer wait on an mbarrier that never
// completes (see mmc_selftest_mbar_timeout).
cudaError_t launch_mbar_timeout_selftest(unsigned long long limit_ns, int* timed_out);

}  // namespace mmc
