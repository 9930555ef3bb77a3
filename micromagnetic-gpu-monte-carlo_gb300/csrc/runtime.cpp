// runtime.cpp -- the C ABI of include/mmc.h: device state of one lattice,
// demag tensor build and cache, sweeps (captured in CUDA graphs) and the
// temperature-stage loop of the reference's main() (src/main.cu:801-1139).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <string>
#include <sys/stat.h>
#include <dirent.h>
#include <vector>

#include "coef.h"
#include "host_common.h"
#include "mmc_internal.h"

namespace mmc {
const char* last_error_cstr();
}

using namespace mmc;

namespace {

const double kB = 1.3806488e-23;  // src/constant.h:22

double pi_of(const mmc_config* c) { return c->use_reference_pi ? 3.14159265358 : 3.14159265358979323846; }

#define CU(x)                                                                               \
  do {                                                                                      \
    cudaError_t e_ = (x);                                                                   \
    if (e_ != cudaSuccess)                                                                  \
      return fail(e_ == cudaErrorMemoryAllocation ? MMC_ERR_OOM : MMC_ERR_CUDA,             \
                  std::string(#x) + ": " + cudaGetErrorString(e_));                         \
  } while (0)

#define TRY(x)                    \
  do {                            \
    int s_ = (x);                 \
    if (s_ != MMC_OK) return s_;  \
  } while (0)

// ------------------------------------------------------------------ FFT plans
struct PlanHost {
  FftPlan p{};
  double2* d64 = nullptr;
  float2* d32 = nullptr;
};

void unit_root(long long j, long long N, double* c, double* s) {
  // exp(-2 pi i j / N) from long double trigonometry on the reduced angle
  j %= N;
  if (j < 0) j += N;
  const long double pi = 3.141592653589793238462643383279502884L;
  long double a = 2.0L * pi * (long double)j / (long double)N;
  *c = (double)cosl(a);
  *s = (double)-sinl(a);
}

// An initial state read from an OVF file as unit vectors: files that store
// the magnetisation M in A/m (OOMMF's usual output) or slightly unnormalised
// m are scaled to |m| = 1; vectors already of unit length to 1e-6 are kept
// as they are (bit for bit).  A zero vector (a vacuum cell) has no direction
// and is an error: every cell of this model is magnetic.
int unit_vectors(double* m3, long long n, const char* path) {
  for (long long i = 0; i < n; ++i) {
    double& x = m3[i];
    double& y = m3[n + i];
    double& z = m3[2 * n + i];
    const double r = std::sqrt(x * x + y * y + z * z);
    if (!(r > 0) || !std::isfinite(r))
      return fail(MMC_ERR_IO, std::string(path) + ": cell " + std::to_string(i) +
                                  " has no magnetisation direction (zero or non-finite vector)");
    if (std::fabs(r - 1.0) > 1e-6) {
      x /= r;
      y /= r;
      z /= r;
    }
  }
  return MMC_OK;
}

// The transform grid's length for a tensor-grid length t: an open axis of
// 2n - 1 > 16 is padded on to the next power of two when that has a
// warp-level transform that every engine takes (32 .. 256); lines of up to 16
// take the per-thread transforms as they are.  Lengths whose power of two
// would be 512 or 1024 (served by the pass kernels' wide transforms only, not
// by the film engine or the batched row kernel) stay as they are when the
// mixed-radix transforms have a plan for them, and are padded only when they
// have a prime factor above FFT_MAX_RADIX or too many factors.
bool has_mixed_radix_plan(int t) {
  int m = t, stages = 0;
  while (m % 2 == 0) m /= 2, ++stages;
  for (int f = 3; m > 1 && f <= FFT_MAX_RADIX; f += 2)
    while (m % f == 0) m /= f, ++stages;
  return m == 1 && stages <= FFT_MAX_STAGES;
}

int transform_len(int t, bool open) {
  if (!open || t <= 16) return t;
  int p = 1;
  while (p < t) p *= 2;
  if (p > 1024) return t;
  if (p <= 256) return p;
  return has_mixed_radix_plan(t) ? t : p;
}

int make_plan(int n, PlanHost* ph) {
  FftPlan& p = ph->p;
  p = FftPlan{};
  p.n = n;
  std::vector<int> rad;
  int m = n;
  while (m % 4 == 0) rad.push_back(4), m /= 4;
  while (m % 2 == 0) rad.push_back(2), m /= 2;
  for (int f = 3; m > 1 && f <= FFT_MAX_RADIX; f += 2)
    while (m % f == 0) rad.push_back(f), m /= f;
  if (m > 1)
    return fail(MMC_ERR_UNSUPPORTED, "FFT length " + std::to_string(n) + " has a prime factor above " +
                                         std::to_string(FFT_MAX_RADIX));
  if ((int)rad.size() > FFT_MAX_STAGES) return fail(MMC_ERR_UNSUPPORTED, "FFT length has too many factors");
  std::vector<double> tw;
  int ns = 1;
  for (size_t s = 0; s < rad.size(); ++s) {
    int R = rad[s];
    p.radix[s] = R;
    p.ns[s] = ns;
    p.dnb[s] = FastDiv((uint32_t)(n / R));
    p.dns[s] = FastDiv((uint32_t)ns);
    p.tw_off[s] = (int)(tw.size() / 2);
    for (int t = 1; t < R; ++t)
      for (int k = 0; k < ns; ++k) {
        double c, sn;
        unit_root((long long)t * k, (long long)ns * R, &c, &sn);
        tw.push_back(c);
        tw.push_back(sn);
      }
    p.root_off[s] = (int)(tw.size() / 2);
    if (R != 2 && R != 3 && R != 4)
      for (int q = 0; q < R; ++q) {
        double c, sn;
        unit_root(q, R, &c, &sn);
        tw.push_back(c);
        tw.push_back(sn);
      }
    ns *= R;
  }
  p.nstages = (int)rad.size();
  // warp-level transform for power-of-two lengths 32 .. 1024: n = A * B
  p.warp_a = p.warp_b = 0;
  p.full_off = 0;
  p.dn = FastDiv((uint32_t)n);
  const int wa[6][3] = {{1024, 32, 32}, {512, 32, 16}, {256, 16, 16}, {128, 16, 8}, {64, 8, 8}, {32, 8, 4}};
  for (const auto& w : wa)
    if (n == w[0]) {
      p.warp_a = w[1];
      p.warp_b = w[2];
    }
  // all n roots exp(-2 pi i j / n) for the warp-level transforms and for the
  // per-thread transforms of short lines (n <= 16)
  if (p.warp_a || n <= 16) {
    p.full_off = (int)(tw.size() / 2);
    for (int j = 0; j < n; ++j) {
      double c, sn;
      unit_root(j, n, &c, &sn);
      tw.push_back(c);
      tw.push_back(sn);
    }
  }
  p.tw_total = (int)(tw.size() / 2);
  size_t cnt = tw.size() / 2;
  if (cnt == 0) cnt = 1, tw.push_back(1.0), tw.push_back(0.0);
  std::vector<float> tw32(tw.size());
  for (size_t i = 0; i < tw.size(); ++i) tw32[i] = (float)tw[i];
  CU(cudaMalloc(&ph->d64, cnt * sizeof(double2)));
  CU(cudaMalloc(&ph->d32, cnt * sizeof(float2)));
  CU(cudaMemcpy(ph->d64, tw.data(), cnt * sizeof(double2), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(ph->d32, tw32.data(), cnt * sizeof(float2), cudaMemcpyHostToDevice));
  p.tw64 = ph->d64;
  p.tw32 = ph->d32;
  return MMC_OK;
}

void free_plan(PlanHost* ph) {
  if (ph->d64) cudaFree(ph->d64);
  if (ph->d32) cudaFree(ph->d32);
  ph->d64 = nullptr;
  ph->d32 = nullptr;
}

size_t smem_limit() { return 220 * 1024; }  // below the 227 KB opt-in limit of a CTA

// Shared memory of an x pass with r rows per CTA, of a column pass with tx
// columns per CTA (bytes).
size_t x_pass_smem(const FftPlan& px, int r, size_t csize) {
  if (px.warp_a)  // k_x_forward_w / k_x_inverse_w: the roots and 2 r padded lines
    return ((size_t)px.n + 2 * (size_t)r * (px.n + px.warp_a)) * csize;
  return ((size_t)((px.tw_total + 1) & ~1) + 2 * (size_t)r * 2 * px.n) * csize;
}
// (lean: the in-place form, which exists for warp-shaped lengths only and
// holds the tile once without a K^ tile)
size_t col_pass_smem(const FftPlan& p, int tx, size_t csize, bool lean = false) {
  const size_t tw = (size_t)((p.tw_total + 1) & ~1), lines = (size_t)3 * tx * col_line_stride(p, csize);
  if (lean && p.warp_a) return (tw + lines) * csize;
  // the pass reads K^ from global memory when its tile would not fit
  const size_t staged = (tw + 2 * lines + 6 * (size_t)p.n * tx) * csize;
  return staged <= smem_limit() ? staged : (tw + 2 * lines) * csize;
}

// Launch shapes for `nrep` replicas.  The warp-level FFT gives each warp
// 32 / B lines, so a CTA takes enough rows / columns to keep all its warps
// busy, and column tiles are widened to whole 32-byte sectors when there are
// enough CTAs to cover the SMs twice.
// threads of a column pass: enough warps for the lines of one tile (3
// components x tx columns)
int col_threads_for(const Geom& g, const FftPlan& py, const FftPlan& pz, int tx, int tx_z) {
  auto threads_for = [&](const FftPlan& p, int t) {
    if (!p.warp_a) return 256;
    const int lines_per_warp = 32 / p.warp_b;
    const int warps = (3 * t + lines_per_warp - 1) / lines_per_warp;
    return std::max(64, std::min(512, 32 * warps));
  };
  return g.nzp == 1 ? threads_for(py, tx) : std::max(threads_for(py, tx), threads_for(pz, tx_z));
}

DemagTuning choose_tuning(const Geom& g, const FftPlan& px, const FftPlan& py, const FftPlan& pz, size_t csize,
                          int nsm, int nrep) {
  DemagTuning t;
  const long long rows = (long long)g.ny * g.nz;
  const long long want = 2LL * nsm;
  auto xsm = [&](int r) { return x_pass_smem(px, r, csize); };
  t.x_threads = px.n >= 512 ? 256 : 128;
  int r = 1;
  if (px.warp_a) {
    const int lines = (t.x_threads / 32) * (32 / px.warp_b);  // lines the warps take in one round
    r = std::max(1, lines / 2);
  } else {
    r = 4;
  }
  while (r > 1 && ((rows + r - 1) / r) * nrep < want) r /= 2;
  while (r > 1 && xsm(r) > 96 * 1024) r /= 2;
  t.x_rows_per_cta = r;
  // in-place column passes reading K^ from global memory for the long
  // warp-shaped lines, where the copies of the tile and of K^ would leave room
  // for one column per CTA (the autotuner tries both forms)
  t.col_lean = py.warp_a != 0 && py.n >= 512 ? 1 : 0;
  // shared memory of a column pass: the in-place form holds the tile once,
  // the other twice plus the K^ tile when the pass multiplies
  auto csm = [&](const FftPlan& p, int tx, bool mul) {
    const size_t tw = (size_t)((p.tw_total + 1) & ~1), lines = (size_t)3 * tx * col_line_stride(p, csize);
    if (t.col_lean && p.warp_a) return (tw + lines) * csize;
    const size_t staged = (tw + 2 * lines + (mul ? 6 * (size_t)p.n * tx : 0)) * csize;
    return staged <= smem_limit() ? staged : (tw + 2 * lines) * csize;  // K^ from global memory
  };
  auto pick = [&](const FftPlan& p, int planes, bool mul) {
    // short lines (a few padded z layers) take wider tiles, up to 64 columns
    int tx = 8;
    while (tx < 64 && tx * p.n < 1024) tx *= 2;
    while (tx > 1 && (((long long)(g.hx + tx - 1) / tx) * planes * nrep < want || csm(p, tx, mul) > 96 * 1024))
      tx /= 2;
    while (tx > 1 && csm(p, tx, mul) > smem_limit()) tx /= 2;
    return tx;
  };
  t.col_tx = pick(py, g.nzp == 1 ? 1 : g.nz, g.nzp == 1);
  t.col_tx_z = pick(pz, g.nyp, true);
  t.col_threads = col_threads_for(g, py, pz, t.col_tx, t.col_tx_z);
  // FP32 with at least 8 x 256^2 trials per launch (batches of 8 films, a
  // 512x512x8 slab): the vectorised per-colour sweep, measured faster there;
  // smaller lattices and FP64 keep the scalar form (the autotuner tries every
  // form)
  t.mc_form = csize == 8 && (long long)nrep * g.n >= 8LL * 65536 && mc_quad_eligible(g) ? MC_FORM_QUAD
                                                                                      : MC_FORM_SCALAR;
  t.fft_inline = 0;
  return t;
}


}  // namespace

// =================================================================== handle
struct mmc_handle {
  mmc_config cfg;
  int device = 0;
  int prec = 32;
  size_t tsize = 4;
  Geom g{};
  cudaStream_t st = nullptr;      // where the handle's work is enqueued (st_own or the caller's)
  cudaStream_t st_own = nullptr;  // created with the handle, destroyed with it
  PlanHost px, py, pz;
  DemagTuning tun{};
  void* m = nullptr;     // 3n T
  void* h = nullptr;     // 3n T, dimensionless demag field K*m
  void* spec = nullptr;  // 3*nspec complex T
  void* khat = nullptr;  // 6*nspec complex T
  void* coef = nullptr;  // McCoef<T> in device memory
  EnCoef* ecoef = nullptr;
  double* partials = nullptr;
  int npartials = 0;
  double* red = nullptr;     // NQ doubles, device
  double* red_host = nullptr;  // NQ doubles, pinned
  unsigned long long* acc = nullptr;
  SweepCounters* ctr = nullptr;
  double* stage64 = nullptr;  // 3n doubles, device (host <-> device staging)
  double* field64 = nullptr;  // 3n doubles, device
  bool demag_built = false;
  double k0[6] = {0, 0, 0, 0, 0, 0};
  std::vector<double> tensor;  // 6*tnp on the tensor grid (txp, typ, tzp), x fastest
  std::atomic<int> stop{0};
  unsigned long long proposed = 0;
  unsigned long long acc_base = 0;
  // graph of `graph_sweeps` sweeps
  cudaGraphExec_t gexec = nullptr;
  int graph_sweeps = 0;
  long long seed = 0;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  double last_run_ms = 0;
  // persistent film engine
  int engine = MMC_ENGINE_KERNELS;
  int fused_band = 0;
  int fused_blocks = 0;
  GridBarrier* bar = nullptr;
  void* hsym = nullptr;      // 3n T, symmetrised demag field of the gradient (allocated on first use)
  double* relax_p = nullptr;  // 3n doubles, relaxation direction
  double* relax_s = nullptr;  // 3n doubles, last relaxation step
  void* m2 = nullptr;     // film engine: second copy of m (3n T)
  void* spec2 = nullptr;  // film engine: second spectrum (3*nspec complex T)
  int nsm = 0;
};

namespace {

int sync_check(mmc_handle* h) {
  CU(cudaStreamSynchronize(h->st));
  return MMC_OK;
}

int set_dev(mmc_handle* h) {
  CU(cudaSetDevice(h->device));
  return MMC_OK;
}

McParams make_mc_params(const mmc_config& c, const double k0[6], long long seed) {
  McParams p;
  p.aex = c.Aex;
  p.dind = c.Dind;
  p.ku1 = c.Ku1;
  p.ms = c.ms;
  p.b[0] = c.Bextx;
  p.b[1] = c.Bexty;
  p.b[2] = c.Bextz;
  double un = std::sqrt(c.anisUx * c.anisUx + c.anisUy * c.anisUy + c.anisUz * c.anisUz);
  p.u[0] = un > 0 ? c.anisUx / un : 0;
  p.u[1] = un > 0 ? c.anisUy / un : 0;
  p.u[2] = un > 0 ? c.anisUz / un : 0;
  p.d[0] = c.dx;
  p.d[1] = c.dy;
  p.d[2] = c.dz;
  p.v = c.dx * c.dy * c.dz;
  p.mu0 = 4e-7 * pi_of(&c);
  for (int q = 0; q < 6; ++q) p.k0[q] = c.cal_demag_flag ? k0[q] : 0.0;
  p.demag = c.cal_demag_flag != 0;
  p.key0 = (uint32_t)((uint64_t)seed & 0xffffffffu);
  p.key1 = (uint32_t)((uint64_t)seed >> 32);
  return p;
}

template <typename T>
McCoef<T> make_mc_coef(const mmc_handle* h, double T_K) {
  return mc_coef_from<T>(make_mc_params(h->cfg, h->k0, h->seed), T_K);
}

int upload_coef(mmc_handle* h, double T_K) {
  if (h->prec == 32) {
    McCoef<float> k = make_mc_coef<float>(h, T_K);
    CU(cudaMemcpyAsync(h->coef, &k, sizeof k, cudaMemcpyHostToDevice, h->st));
  } else {
    McCoef<double> k = make_mc_coef<double>(h, T_K);
    CU(cudaMemcpyAsync(h->coef, &k, sizeof k, cudaMemcpyHostToDevice, h->st));
  }
  // the source is a stack object: wait for the copy before it goes out of scope
  CU(cudaStreamSynchronize(h->st));
  return MMC_OK;
}

EnCoef make_en_coef(const mmc_handle* h) {
  const mmc_config& c = h->cfg;
  EnCoef e;
  const double V = c.dx * c.dy * c.dz;
  const double d[3] = {c.dx, c.dy, c.dz};
  for (int a = 0; a < 3; ++a) e.aexV_d2[a] = c.Aex * V / (d[a] * d[a]);
  e.dV_2d[0] = c.Dind * V / (2.0 * d[0]);
  e.dV_2d[1] = c.Dind * V / (2.0 * d[1]);
  e.kuV = c.Ku1 * V;
  double un = std::sqrt(c.anisUx * c.anisUx + c.anisUy * c.anisUy + c.anisUz * c.anisUz);
  e.u[0] = un > 0 ? c.anisUx / un : 0;
  e.u[1] = un > 0 ? c.anisUy / un : 0;
  e.u[2] = un > 0 ? c.anisUz / un : 0;
  e.msVB[0] = c.ms * V * c.Bextx;
  e.msVB[1] = c.ms * V * c.Bexty;
  e.msVB[2] = c.ms * V * c.Bextz;
  const double mu0 = 4e-7 * pi_of(&c);
  e.demag = c.cal_demag_flag ? 0.5 * mu0 * c.ms * c.ms * V : 0.0;
  return e;
}

HCoef make_h_coef(const mmc_handle* h) {
  const mmc_config& c = h->cfg;
  HCoef k;
  const double mu0 = 4e-7 * pi_of(&c);
  const double d[3] = {c.dx, c.dy, c.dz};
  for (int a = 0; a < 3; ++a) k.ex_d2[a] = 2.0 * c.Aex / (mu0 * c.ms) / (d[a] * d[a]);
  k.dm_2d[0] = 2.0 * c.Dind / (mu0 * c.ms) / (2.0 * d[0]);
  k.dm_2d[1] = 2.0 * c.Dind / (mu0 * c.ms) / (2.0 * d[1]);
  k.an = 2.0 * c.Ku1 / (mu0 * c.ms);
  double un = std::sqrt(c.anisUx * c.anisUx + c.anisUy * c.anisUy + c.anisUz * c.anisUz);
  k.u[0] = un > 0 ? c.anisUx / un : 0;
  k.u[1] = un > 0 ? c.anisUy / un : 0;
  k.u[2] = un > 0 ? c.anisUz / un : 0;
  k.b[0] = c.Bextx / mu0;
  k.b[1] = c.Bexty / mu0;
  k.b[2] = c.Bextz / mu0;
  k.ms = c.cal_demag_flag ? c.ms : 0.0;
  return k;
}

cudaError_t demag(mmc_handle* h) {
  if (h->prec == 32)
    return launch_demag<float>(h->g, h->px.p, h->py.p, h->pz.p, h->tun, (const float*)h->m, (float*)h->h, h->spec,
                               h->khat, h->st);
  return launch_demag<double>(h->g, h->px.p, h->py.p, h->pz.p, h->tun, (const double*)h->m, (double*)h->h, h->spec,
                              h->khat, h->st);
}

cudaError_t mc_color(mmc_handle* h, int color) {
  if (h->prec == 32)
    return launch_mc<float>(h->g, (const McCoef<float>*)h->coef, (float*)h->m, (const float*)h->h, h->ctr, color,
                            h->acc, h->st, 1, h->tun.mc_form);
  return launch_mc<double>(h->g, (const McCoef<double>*)h->coef, (double*)h->m, (const double*)h->h, h->ctr, color,
                           h->acc, h->st, 1, h->tun.mc_form);
}

// Enqueues one full sweep: demag refresh, every colour, counter advance.
cudaError_t enqueue_sweep(mmc_handle* h) {
  cudaError_t e;
  if (h->cfg.cal_demag_flag) {
    e = demag(h);
    if (e != cudaSuccess) return e;
  }
  e = mc_color(h, -1);
  if (e != cudaSuccess) return e;
  return launch_advance(h->ctr, 1, h->st);
}

int ensure_graph(mmc_handle* h, int nsw) {
  if (h->gexec && h->graph_sweeps == nsw) return MMC_OK;
  if (h->gexec) {
    cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
  }
  cudaGraph_t graph;
  CU(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  for (int s = 0; s < nsw && e == cudaSuccess; ++s) e = enqueue_sweep(h);
  cudaError_t e2 = cudaStreamEndCapture(h->st, &graph);
  if (e != cudaSuccess || e2 != cudaSuccess) cudaGetLastError();  // do not leak the capture error to later calls
  if (e != cudaSuccess) return fail(MMC_ERR_CUDA, std::string("sweep capture: ") + cudaGetErrorString(e));
  if (e2 != cudaSuccess) return fail(MMC_ERR_CUDA, std::string("sweep capture end: ") + cudaGetErrorString(e2));
  e = cudaGraphInstantiate(&h->gexec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return fail(MMC_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  h->graph_sweeps = nsw;
  return MMC_OK;
}

int build_demag_impl(mmc_handle* h, const char* cache_dir);

int ensure_demag(mmc_handle* h) {
  if (!h->cfg.cal_demag_flag || h->demag_built) return MMC_OK;
  return build_demag_impl(h, h->cfg.tensor_cache);
}

// The persistent film engine: chunks of at most 1024 sweeps per cooperative
// launch; a stop request is honoured between chunks, a barrier timeout inside
// the kernel is reported as MMC_ERR_TIMEOUT.
template <typename T>
cudaError_t fused_chunk(mmc_handle* h, long long stage, long long sweep0, int ns,
                        unsigned long long* tbuf = nullptr) {
  FusedArgs<T> a;
  a.coef = (const McCoef<T>*)h->coef;
  a.m = (T*)h->m;
  a.m2 = (T*)h->m2;
  a.h = (T*)h->h;
  a.spec = h->spec;
  a.spec2 = h->spec2;
  a.khat = h->khat;
  a.acc = h->acc;
  a.bar = h->bar;
  a.tbuf = tbuf;
  a.stage = (uint32_t)stage;
  a.sweep0 = (uint32_t)sweep0;
  a.nsweeps = ns;
  a.band = h->fused_band;
  cudaError_t e = launch_fused2d<T>(h->g, h->px.p, h->py.p, a, h->fused_blocks, h->st);
  // an odd sweep count leaves the result in the second copy
  if (e == cudaSuccess && (ns & 1))
    e = cudaMemcpyAsync(h->m, h->m2, 3 * (size_t)h->g.n * sizeof(T), cudaMemcpyDeviceToDevice, h->st);
  return e;
}

int run_fused(mmc_handle* h, long long stage, long long sweep0, long long nsweeps) {
  CU(cudaEventRecord(h->ev[0], h->st));
  long long done = 0;
  while (done < nsweeps) {
    if (h->stop.load()) return fail(MMC_ERR_INTERRUPTED, "stop requested");
    const int ns = (int)std::min<long long>(1024, nsweeps - done);
    CU(h->prec == 32 ? fused_chunk<float>(h, stage, sweep0 + done, ns)
                     : fused_chunk<double>(h, stage, sweep0 + done, ns));
    done += ns;
    if ((done / 1024) % 8 == 0 || done == nsweeps) {
      CU(cudaStreamSynchronize(h->st));
      std::vector<unsigned char> hb(grid_barrier_bytes());
      CU(cudaMemcpy(hb.data(), h->bar, hb.size(), cudaMemcpyDeviceToHost));
      if (grid_barrier_error(reinterpret_cast<const GridBarrier*>(hb.data())))
        return fail(MMC_ERR_TIMEOUT, "grid barrier wait ran out of its budget in the film engine");
    }
  }
  CU(cudaEventRecord(h->ev[1], h->st));
  CU(cudaStreamSynchronize(h->st));
  float ms = 0;
  CU(cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]));
  h->last_run_ms = ms;
  h->proposed += (unsigned long long)nsweeps * (unsigned long long)h->g.n;
  return MMC_OK;
}

// Picks the film engine's band (rows per CTA) and CTA count: the smallest band
// from the preference list whose grid is co-resident.
int setup_engine(mmc_handle* h, int nsm) {
  const mmc_config& c = h->cfg;
  const Geom& g = h->g;
  // films with demag and two colours whose m rows are whole 16-byte chunks
  const bool eligible = c.cal_demag_flag && g.nz == 1 && g.nzp == 1 && g.ncolors == 2 &&
                        ((size_t)g.nx * h->tsize) % 16 == 0 && g.ny >= 1 && h->px.p.warp_a != 32 &&
                        h->py.p.warp_a != 32;
  if (c.sweep_engine == MMC_ENGINE_KERNELS || (c.sweep_engine == MMC_ENGINE_AUTO && !eligible)) {
    h->engine = MMC_ENGINE_KERNELS;
    return MMC_OK;
  }
  if (!eligible)
    return fail(MMC_ERR_UNSUPPORTED,
                "the fused engine needs a film (nz = 1), demag on, an even or open lattice, nx * sizeof(real) "
                "a multiple of 16 bytes and padded sides other than 512 and 1024");
  int optin = 48 * 1024;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
  std::vector<int> bands;
  if (c.fused_band > 0) bands.push_back(c.fused_band);
  else bands = {2, 1, 3, 4, 6, 8, 12, 16, 24, 32, 48, 60};
  for (int b : bands) {
    const size_t smem = h->prec == 32 ? fused2d_smem_bytes<float>(g, h->px.p, h->py.p, b)
                                      : fused2d_smem_bytes<double>(g, h->px.p, h->py.p, b);
    if (smem > (size_t)optin) continue;
    int per_sm = 0;
    cudaError_t e = h->prec == 32 ? fused2d_blocks_per_sm<float>(g, h->px.p, h->py.p, b, &per_sm)
                                  : fused2d_blocks_per_sm<double>(g, h->px.p, h->py.p, b, &per_sm);
    if (e != cudaSuccess) return fail(MMC_ERR_CUDA, std::string("occupancy query: ") + cudaGetErrorString(e));
    const int blocks = (g.ny + b - 1) / b;
    if (per_sm > 0 && blocks <= per_sm * nsm) {
      h->engine = MMC_ENGINE_FUSED;
      h->fused_band = b;
      h->fused_blocks = blocks;
      void* p = nullptr;
      CU(cudaMalloc(&p, grid_barrier_bytes()));
      CU(cudaMemset(p, 0, grid_barrier_bytes()));
      h->bar = (GridBarrier*)p;
      CU(cudaMalloc(&h->m2, 3 * (size_t)g.n * h->tsize));
      CU(cudaMalloc(&h->spec2, 3 * (size_t)g.nspec * 2 * h->tsize));
      return MMC_OK;
    }
  }
  if (c.sweep_engine == MMC_ENGINE_FUSED)
    return fail(MMC_ERR_UNSUPPORTED, "no film-engine band fits this lattice on this device");
  h->engine = MMC_ENGINE_KERNELS;
  return MMC_OK;
}

// Runs `nsweeps` sweeps with counters (stage, sweep0); graph replays for the bulk.
int run_sweeps_impl(mmc_handle* h, double T_K, long long stage, long long sweep0, long long nsweeps) {
  if (nsweeps <= 0) return MMC_OK;
  TRY(ensure_demag(h));
  TRY(upload_coef(h, T_K));
  SweepCounters c0{(uint32_t)stage, (uint32_t)sweep0};
  CU(cudaMemcpyAsync(h->ctr, &c0, sizeof c0, cudaMemcpyHostToDevice, h->st));
  CU(cudaStreamSynchronize(h->st));
  if (h->engine == MMC_ENGINE_FUSED) return run_fused(h, stage, sweep0, nsweeps);
  const int G = 64;
  long long done = 0;
  CU(cudaEventRecord(h->ev[0], h->st));
  if (nsweeps >= G) {
    TRY(ensure_graph(h, G));
    while (nsweeps - done >= G) {
      if (h->stop.load()) return fail(MMC_ERR_INTERRUPTED, "stop requested");
      CU(cudaGraphLaunch(h->gexec, h->st));
      done += G;
      // bound the amount of queued work so a stop request takes effect quickly
      if ((done / G) % 16 == 0) CU(cudaStreamSynchronize(h->st));
    }
  }
  for (; done < nsweeps; ++done) CU(enqueue_sweep(h));
  CU(cudaEventRecord(h->ev[1], h->st));
  CU(cudaStreamSynchronize(h->st));
  float ms = 0;
  CU(cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]));
  h->last_run_ms = ms;
  h->proposed += (unsigned long long)nsweeps * (unsigned long long)h->g.n;
  return MMC_OK;
}

int profile_sweeps_impl(mmc_handle* h, double T_K, long long stage, long long sweep0, long long nsweeps,
                        double out[3]) {
  TRY(ensure_demag(h));
  TRY(upload_coef(h, T_K));
  SweepCounters c0{(uint32_t)stage, (uint32_t)sweep0};
  CU(cudaMemcpyAsync(h->ctr, &c0, sizeof c0, cudaMemcpyHostToDevice, h->st));
  CU(cudaStreamSynchronize(h->st));
  double tdem = 0, tmc = 0;
  cudaEvent_t a = h->ev[0], b = h->ev[1], c = h->ev[2], t0 = h->ev[3];
  CU(cudaEventRecord(t0, h->st));
  for (long long s = 0; s < nsweeps; ++s) {
    CU(cudaEventRecord(a, h->st));
    if (h->cfg.cal_demag_flag) CU(demag(h));
    CU(cudaEventRecord(b, h->st));
    CU(mc_color(h, -1));
    CU(cudaEventRecord(c, h->st));
    CU(launch_advance(h->ctr, 1, h->st));
    CU(cudaEventSynchronize(c));
    float x = 0, y = 0;
    CU(cudaEventElapsedTime(&x, a, b));
    CU(cudaEventElapsedTime(&y, b, c));
    tdem += x;
    tmc += y;
  }
  CU(cudaEventRecord(b, h->st));
  CU(cudaStreamSynchronize(h->st));
  float tot = 0;
  CU(cudaEventElapsedTime(&tot, t0, b));
  out[0] = tdem;
  out[1] = tmc;
  out[2] = tot;
  h->proposed += (unsigned long long)nsweeps * (unsigned long long)h->g.n;
  return MMC_OK;
}

// Squared switch distance of the far-field tensor terms (0 = off).
double far_r2(const mmc_config& c) {
  if (c.tensor_far_radius <= 0) return 0.0;
  const double d = std::max(c.dx, std::max(c.dy, c.dz)) * (double)c.tensor_far_radius;
  return d * d;
}

std::string cache_name(const mmc_handle* h) {
  char b[256];
  std::snprintf(b, sizeof b, "cache_%d_%d_%d-%g_%g_%g-%d_%d_%d", h->g.txp, h->g.typ, h->g.tzp, h->cfg.dx,
                h->cfg.dy, h->cfg.dz, h->cfg.pbc_x, h->cfg.pbc_y, h->cfg.pbc_z);
  std::string name = b;
  // a tensor with far-field terms is not the reference's: keep it apart
  if (h->cfg.tensor_far_radius > 0) name += "_far" + std::to_string(h->cfg.tensor_far_radius);
  return name + ".ovf";
}

bool dir_exists(const std::string& d) {
  struct stat sb;
  return !d.empty() && stat(d.c_str(), &sb) == 0 && S_ISDIR(sb.st_mode);
}

std::string join(const std::string& d, const std::string& f) {
  if (d.empty()) return f;
  return d.back() == '/' ? d + f : d + "/" + f;
}

// Tensor cache in the reference's raw format (src/main.cu:427-455, 548-572):
// 6 blocks xx,xy,xz,yy,yz,zz of txp*typ*tzp doubles (the tensor grid), z fastest / x slowest.
bool cache_load(mmc_handle* h, const std::string& path) {
  std::ifstream in(path, std::ios::binary);
  if (!in) return false;
  const Geom& g = h->g;
  std::vector<double> raw(6 * (size_t)g.tnp);
  in.read(reinterpret_cast<char*>(raw.data()), (std::streamsize)(raw.size() * sizeof(double)));
  if (!in || in.gcount() != (std::streamsize)(raw.size() * sizeof(double))) return false;
  h->tensor.assign(6 * (size_t)g.tnp, 0.0);
  for (int c = 0; c < 6; ++c)
    for (int x = 0; x < g.txp; ++x)
      for (int y = 0; y < g.typ; ++y)
        for (int z = 0; z < g.tzp; ++z)
          h->tensor[c * g.tnp + x + (long long)g.txp * (y + (long long)g.typ * z)] =
              raw[c * g.tnp + z + (long long)g.tzp * (y + (long long)g.typ * x)];
  return true;
}

bool cache_save(const mmc_handle* h, const std::string& path) {
  const Geom& g = h->g;
  std::vector<double> raw(6 * (size_t)g.tnp);
  for (int c = 0; c < 6; ++c)
    for (int x = 0; x < g.txp; ++x)
      for (int y = 0; y < g.typ; ++y)
        for (int z = 0; z < g.tzp; ++z)
          raw[c * g.tnp + z + (long long)g.tzp * (y + (long long)g.typ * x)] =
              h->tensor[c * g.tnp + x + (long long)g.txp * (y + (long long)g.typ * z)];
  std::ofstream out(path, std::ios::binary | std::ios::trunc);
  if (!out) return false;
  out.write(reinterpret_cast<const char*>(raw.data()), (std::streamsize)(raw.size() * sizeof(double)));
  return (bool)out;
}

int build_demag_impl(mmc_handle* h, const char* cache_dir) {
  TRY(set_dev(h));
  const Geom& g = h->g;
  const mmc_config& c = h->cfg;
  std::string dir = cache_dir ? cache_dir : "";
  std::string path = dir.empty() ? "" : join(dir, cache_name(h));
  bool loaded = !path.empty() && cache_load(h, path);
  double* k6 = nullptr;   // the tensor grid
  double* k6f = nullptr;  // the transform grid, when it differs
  double2* spec64 = nullptr;
  CU(cudaMalloc(&k6, 6 * (size_t)g.tnp * sizeof(double)));
  int status = MMC_OK;
  do {
    if (loaded) {
      cudaError_t e = cudaMemcpy(k6, h->tensor.data(), 6 * (size_t)g.tnp * sizeof(double), cudaMemcpyHostToDevice);
      if (e != cudaSuccess) {
        status = fail(MMC_ERR_CUDA, cudaGetErrorString(e));
        break;
      }
    } else {
      const int Px = std::max(c.pbc_x, 0), Py = std::max(c.pbc_y, 0), Pz = std::max(c.pbc_z, 0);
      // Each launch adds a slab of x images to every point's running sum; about
      // 1e9 f/g evaluations per launch keeps launches near a second (384 per
      // point and image in the term form, 6 x 972 per 256 points in the node form).
      const double per_px = (double)g.tnp * (2.0 * Py + 1) * (2.0 * Pz + 1) * (c.tensor_sum == 1 ? 23.0 : 384.0);
      const int slab = std::max(1, (int)(1e9 / per_px));
      for (int px0 = -Px; px0 <= Px; px0 += slab) {
        if (h->stop.load()) {
          status = fail(MMC_ERR_INTERRUPTED, "stop requested during the tensor build");
          break;
        }
        const int px1 = std::min(Px, px0 + slab - 1);
        cudaError_t e = launch_newell(g, c.dx, c.dy, c.dz, Px, Py, Pz, pi_of(&c), k6, px0, px1, px1 == Px, h->st,
                                      far_r2(c), c.tensor_sum);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
        if (e != cudaSuccess) {
          status = fail(MMC_ERR_CUDA, std::string("tensor build: ") + cudaGetErrorString(e));
          break;
        }
      }
      if (status != MMC_OK) break;
      h->tensor.assign(6 * (size_t)g.tnp, 0.0);
      cudaError_t e = cudaMemcpy(h->tensor.data(), k6, 6 * (size_t)g.tnp * sizeof(double), cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) {
        status = fail(MMC_ERR_CUDA, cudaGetErrorString(e));
        break;
      }
      if (!path.empty() && dir_exists(dir)) cache_save(h, path);
    }
    for (int q = 0; q < 6; ++q) h->k0[q] = h->tensor[(size_t)q * g.tnp];
    cudaError_t e = cudaSuccess;
    if (g.np != g.tnp) {  // the tensor on the transform grid
      e = cudaMalloc(&k6f, 6 * (size_t)g.np * sizeof(double));
      if (e == cudaSuccess) e = launch_tensor_rewrap(g, k6, k6f, h->st);
      if (e != cudaSuccess) {
        status = fail(MMC_ERR_CUDA, std::string("tensor re-wrap: ") + cudaGetErrorString(e));
        break;
      }
    }
    e = cudaMalloc(&spec64, 6 * (size_t)g.nspec * sizeof(double2));
    if (e != cudaSuccess) {
      status = fail(MMC_ERR_OOM, "tensor spectrum allocation");
      break;
    }
    DemagTuning tt = h->tun;
    // six-component setup transform: narrower tiles keep shared memory in budget
    while (tt.col_tx > 1 && ((size_t)((h->py.p.tw_total + 1) & ~1) + 2 * 3 * (size_t)tt.col_tx * col_line_stride(h->py.p, sizeof(double2))) *
                                    sizeof(double2) > smem_limit())
      tt.col_tx /= 2;
    while (tt.col_tx_z > 1 && ((size_t)((h->pz.p.tw_total + 1) & ~1) + 2 * 3 * (size_t)tt.col_tx_z * col_line_stride(h->pz.p, sizeof(double2))) *
                                      sizeof(double2) > smem_limit())
      tt.col_tx_z /= 2;
    tt.col_tx = std::min(tt.col_tx, tt.col_tx_z);
    tt.col_tx_z = tt.col_tx;
    e = launch_tensor_fft(g, h->px.p, h->py.p, h->pz.p, tt, k6f ? k6f : k6, spec64, h->st);
    if (e == cudaSuccess) {
      if (h->prec == 32) e = launch_khat_store<float>(6 * g.nspec, spec64, h->khat, h->st);
      else e = launch_khat_store<double>(6 * g.nspec, spec64, h->khat, h->st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    if (e != cudaSuccess) {
      status = fail(MMC_ERR_CUDA, std::string("tensor transform: ") + cudaGetErrorString(e));
      break;
    }
    h->demag_built = true;
  } while (0);
  if (spec64) cudaFree(spec64);
  if (k6f) cudaFree(k6f);
  if (k6) cudaFree(k6);
  return status;
}

int get_m_impl(mmc_handle* h, double* mx, double* my, double* mz) {
  const long long n = h->g.n;
  cudaError_t e = h->prec == 32 ? launch_to_f64<float>(3 * n, (const float*)h->m, h->stage64, h->st)
                                : launch_to_f64<double>(3 * n, (const double*)h->m, h->stage64, h->st);
  CU(e);
  CU(cudaMemcpyAsync(mx, h->stage64, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CU(cudaMemcpyAsync(my, h->stage64 + n, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CU(cudaMemcpyAsync(mz, h->stage64 + 2 * n, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CU(cudaStreamSynchronize(h->st));
  return MMC_OK;
}

int set_m_impl(mmc_handle* h, const double* mx, const double* my, const double* mz) {
  const long long n = h->g.n;
  CU(cudaMemcpyAsync(h->stage64, mx, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
  CU(cudaMemcpyAsync(h->stage64 + n, my, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
  CU(cudaMemcpyAsync(h->stage64 + 2 * n, mz, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
  cudaError_t e = h->prec == 32 ? launch_from_f64<float>(3 * n, h->stage64, (float*)h->m, h->st)
                                : launch_from_f64<double>(3 * n, h->stage64, (double*)h->m, h->st);
  CU(e);
  CU(cudaStreamSynchronize(h->st));
  return MMC_OK;
}

// ------------------------------------------------------------ gradient
// The demag field with the symmetrised tensor, into h->hsym.
int demag_sym(mmc_handle* h) {
  if (!h->hsym) CU(cudaMalloc(&h->hsym, 3 * (size_t)h->g.n * h->tsize));
  CU(h->prec == 32 ? launch_demag_sym<float>(h->g, h->px.p, h->py.p, h->pz.p, h->tun, (const float*)h->m,
                                             (float*)h->hsym, h->spec, h->khat, h->st)
                   : launch_demag_sym<double>(h->g, h->px.p, h->py.p, h->pz.p, h->tun, (const double*)h->m,
                                              (double*)h->hsym, h->spec, h->khat, h->st));
  return MMC_OK;
}

int grad_impl(mmc_handle* h, double* grad, double dparams[7]) {
  TRY(ensure_demag(h));
  const mmc_config& c = h->cfg;
  const bool dm = c.cal_demag_flag != 0;
  if (dm) TRY(demag_sym(h));
  const HCoef k = make_h_coef(h);
  // prefactors of the energy terms at unit Aex, Dind, Ku1 and d/dMs
  EnCoef eu = make_en_coef(h);
  const double V = c.dx * c.dy * c.dz;
  const double d[3] = {c.dx, c.dy, c.dz};
  const double mu0 = 4e-7 * pi_of(&c);
  for (int a = 0; a < 3; ++a) eu.aexV_d2[a] = V / (d[a] * d[a]);
  eu.dV_2d[0] = V / (2.0 * d[0]);
  eu.dV_2d[1] = V / (2.0 * d[1]);
  eu.kuV = V;
  eu.msVB[0] = V * c.Bextx;
  eu.msVB[1] = V * c.Bexty;
  eu.msVB[2] = V * c.Bextz;
  eu.demag = dm ? mu0 * c.ms * V : 0.0;
  const double gscale = -mu0 * c.ms * V;
  double* gdev = grad ? h->field64 : nullptr;
  CU(h->prec == 32 ? launch_grad<float>(h->g, k, eu, gscale, (const float*)h->m, dm ? (const float*)h->hsym : nullptr,
                                        gdev, h->partials, h->npartials, h->red, h->st)
                   : launch_grad<double>(h->g, k, eu, gscale, (const double*)h->m,
                                         dm ? (const double*)h->hsym : nullptr, gdev, h->partials, h->npartials,
                                         h->red, h->st));
  CU(cudaMemcpyAsync(h->red_host, h->red, NQ * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  if (grad) CU(cudaMemcpyAsync(grad, h->field64, 3 * (size_t)h->g.n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  TRY(sync_check(h));
  const double* r = h->red_host;
  dparams[0] = r[0];
  dparams[1] = r[1];
  dparams[2] = r[2];
  dparams[3] = r[3] + r[4];
  for (int a = 0; a < 3; ++a) dparams[4 + a] = -c.ms * V * r[5 + a];
  return MMC_OK;
}

// Projected steepest descent with Barzilai-Borwein steps (see grad.cuh) until
// max |m x H| / Ms < tol or max_iter updates.
int relax_impl(mmc_handle* h, double tol, long long max_iter, long long* iters, double* torque) {
  TRY(ensure_demag(h));
  const size_t n3 = 3 * (size_t)h->g.n;
  if (!h->relax_p) CU(cudaMalloc(&h->relax_p, n3 * sizeof(double)));
  if (!h->relax_s) CU(cudaMalloc(&h->relax_s, n3 * sizeof(double)));
  const bool dm = h->cfg.cal_demag_flag != 0;
  const HCoef k = make_h_coef(h);
  const double inv_ms = 1.0 / h->cfg.ms;
  const double tau0 = 1e-3;
  double tau = tau0, tq = 0;
  long long it = 0;
  for (;; ++it) {
    if (h->stop.load()) return fail(MMC_ERR_INTERRUPTED, "stop requested");
    if (dm) TRY(demag_sym(h));
    CU(h->prec == 32 ? launch_relax_eval<float>(h->g, k, inv_ms, (const float*)h->m,
                                                dm ? (const float*)h->hsym : nullptr, h->relax_p, h->relax_s,
                                                it == 0, h->partials, h->npartials, h->red, h->st)
                     : launch_relax_eval<double>(h->g, k, inv_ms, (const double*)h->m,
                                                 dm ? (const double*)h->hsym : nullptr, h->relax_p, h->relax_s,
                                                 it == 0, h->partials, h->npartials, h->red, h->st));
    CU(cudaMemcpyAsync(h->red_host, h->red, 4 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    TRY(sync_check(h));
    const double ss = h->red_host[0], sy = h->red_host[1], yy = h->red_host[2];
    tq = h->red_host[3];
    if (!std::isfinite(tq) || !std::isfinite(ss + sy + yy))
      return fail(MMC_ERR_INVALID, "relaxation produced a non-finite torque");
    if (tq < tol || it >= max_iter) break;
    if (it > 0) {
      // the long Barzilai-Borwein step s.s / s.y (the short one, s.y / y.y,
      // stalled on annealed films in tests); keep the last step when the
      // curvature estimate is not positive
      const double t = ss / sy;
      (void)yy;
      if (std::isfinite(t) && t > 0) tau = t;
    }
    CU(h->prec == 32 ? launch_relax_update<float>(h->g, (float*)h->m, h->relax_p, tau, h->relax_s, h->st)
                     : launch_relax_update<double>(h->g, (double*)h->m, h->relax_p, tau, h->relax_s, h->st));
  }
  if (iters) *iters = it;
  if (torque) *torque = tq;
  return MMC_OK;
}

int energy_impl(mmc_handle* h, mmc_observables* out) {
  TRY(ensure_demag(h));
  if (h->cfg.cal_demag_flag) CU(demag(h));
  EnCoef e = make_en_coef(h);
  CU(cudaMemcpyAsync(h->ecoef, &e, sizeof e, cudaMemcpyHostToDevice, h->st));
  cudaError_t err =
      h->prec == 32
          ? launch_energy<float>(h->g, h->ecoef, (const float*)h->m, h->cfg.cal_demag_flag ? (const float*)h->h : nullptr,
                                 h->partials, h->npartials, h->red, h->st)
          : launch_energy<double>(h->g, h->ecoef, (const double*)h->m, h->cfg.cal_demag_flag ? (const double*)h->h : nullptr,
                                  h->partials, h->npartials, h->red, h->st);
  CU(err);
  CU(cudaMemcpyAsync(h->red_host, h->red, NQ * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  unsigned long long acc = 0;
  CU(cudaMemcpyAsync(&acc, h->acc, sizeof acc, cudaMemcpyDeviceToHost, h->st));
  CU(cudaStreamSynchronize(h->st));
  const double* r = h->red_host;
  const double n = (double)h->g.n;
  out->e_exchange = r[0];
  out->e_dmi = r[1];
  out->e_anisotropy = r[2];
  out->e_zeeman = r[3];
  out->e_demag = r[4];
  out->e_total = r[0] + r[1] + r[2] + r[3] + r[4];
  out->m[0] = r[5] / n;
  out->m[1] = r[6] / n;
  out->m[2] = r[7] / n;
  out->q = r[8] / (4.0 * 3.14159265358979323846) / (double)h->g.nz;
  out->accepted = acc - h->acc_base;
  out->proposed = h->proposed;
  h->acc_base = acc;
  h->proposed = 0;
  return MMC_OK;
}

void destroy_impl(mmc_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  void* bufs[] = {h->m,   h->h,   h->spec,    h->khat,    h->coef,          h->partials,     h->red,
                  h->acc, h->ctr, h->stage64, h->field64, (void*)h->bar, (void*)h->ecoef, h->m2, h->spec2,
                  h->hsym, h->relax_p, h->relax_s};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (h->red_host) cudaFreeHost(h->red_host);
  for (auto& e : h->ev)
    if (e) cudaEventDestroy(e);
  free_plan(&h->px);
  free_plan(&h->py);
  free_plan(&h->pz);
  if (h->st_own) cudaStreamDestroy(h->st_own);
  delete h;
}

int create_impl(const mmc_config* cfg, int device, mmc_handle** out) {
  *out = nullptr;
  TRY(config_validate(cfg));
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(MMC_ERR_NO_DEVICE, "no CUDA device");
  if (device < 0 || device >= ndev) return fail(MMC_ERR_INVALID, "device index out of range");
  mmc_handle* h = new mmc_handle();
  h->cfg = *cfg;
  h->device = device;
  h->prec = cfg->precision;
  h->tsize = h->prec == 32 ? 4 : 8;
  h->seed = cfg->randomseed < 0 ? (long long)std::time(nullptr) : cfg->randomseed;
  h->cfg.randomseed = h->seed;
  auto bail = [&](int st) {
    std::string msg = last_error_cstr();
    destroy_impl(h);
    fail(st, msg);
    return st;
  };
  if (cudaSetDevice(device) != cudaSuccess) return bail(fail(MMC_ERR_CUDA, "cudaSetDevice failed"));
  Geom& g = h->g;
  g.nx = cfg->nx;
  g.ny = cfg->ny;
  g.nz = cfg->nz;
  // the tensor grid, src/main.cu:254-263
  g.txp = cfg->pbc_x == 0 ? 2 * cfg->nx - 1 : cfg->nx;
  g.typ = cfg->pbc_y == 0 ? 2 * cfg->ny - 1 : cfg->ny;
  g.tzp = cfg->pbc_z == 0 ? 2 * cfg->nz - 1 : cfg->nz;
  g.nxp = transform_len(g.txp, cfg->pbc_x == 0);
  g.nyp = transform_len(g.typ, cfg->pbc_y == 0);
  g.nzp = transform_len(g.tzp, cfg->pbc_z == 0);
  g.hx = g.nxp / 2 + 1;
  g.hxp = g.hx + (g.hx & 1);
  g.per[0] = cfg->pbc_x != 0;
  g.per[1] = cfg->pbc_y != 0;
  g.per[2] = cfg->pbc_z != 0;
  g.ncolors = 2;
  const int dims[3] = {g.nx, g.ny, g.nz};
  for (int a = 0; a < 3; ++a)
    if (g.per[a] && (dims[a] & 1) && dims[a] > 1) g.ncolors = 3;
  g.n = (long long)g.nx * g.ny * g.nz;
  g.np = (long long)g.nxp * g.nyp * g.nzp;
  g.tnp = (long long)g.txp * g.typ * g.tzp;
  g.nspec = (long long)g.hxp * g.nyp * g.nzp;
  g.dnx = FastDiv((uint32_t)g.nx);
  g.dny = FastDiv((uint32_t)g.ny);
  g.dhx = FastDiv((uint32_t)g.hx);
  g.dhxc = FastDiv((uint32_t)((g.nx + 1) / 2));
  int st;
  if (cudaStreamCreateWithFlags(&h->st_own, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(MMC_ERR_CUDA, "stream creation failed"));
  h->st = h->st_own;
  if ((st = make_plan(g.nxp, &h->px)) != MMC_OK) return bail(st);
  if ((st = make_plan(g.nyp, &h->py)) != MMC_OK) return bail(st);
  if ((st = make_plan(g.nzp, &h->pz)) != MMC_OK) return bail(st);
  int nsm = 148, optin = 48 * 1024;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  if (launch_prepare<float>(optin) != cudaSuccess || launch_prepare<double>(optin) != cudaSuccess)
    return bail(fail(MMC_ERR_CUDA, "kernel attribute setup failed"));
  const size_t csize = 2 * h->tsize;
  h->tun = choose_tuning(g, h->px.p, h->py.p, h->pz.p, csize, nsm, 1);
  h->nsm = nsm;
  // shared-memory feasibility of the per-sweep passes
  if (((size_t)((h->px.p.tw_total + 1) & ~1) + 2 * 2 * (size_t)h->px.p.n) * csize > smem_limit() ||
      ((size_t)((h->py.p.tw_total + 1) & ~1) + 2 * 3 * (size_t)col_line_stride(h->py.p, csize)) * csize > smem_limit() ||
      ((size_t)((h->pz.p.tw_total + 1) & ~1) + 2 * 3 * (size_t)col_line_stride(h->pz.p, csize)) * csize > smem_limit() ||
      ((size_t)((h->px.p.tw_total + 1) & ~1) + 2 * 3 * (size_t)h->px.p.n) * 16 > smem_limit())
    return bail(fail(MMC_ERR_UNSUPPORTED, "padded lattice dimension too large for the shared-memory FFT"));
  auto alloc = [&](void** p, size_t bytes) -> int {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return fail(MMC_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return MMC_OK;
  };
  h->npartials = energy_partials_count(g);
  if ((st = alloc(&h->m, 3 * g.n * h->tsize)) != MMC_OK) return bail(st);
  if ((st = alloc(&h->h, 3 * g.n * h->tsize)) != MMC_OK) return bail(st);
  if (cfg->cal_demag_flag) {
    if ((st = alloc(&h->spec, 3 * g.nspec * csize)) != MMC_OK) return bail(st);
    if ((st = alloc(&h->khat, 6 * g.nspec * csize)) != MMC_OK) return bail(st);
  }
  if ((st = alloc(&h->coef, sizeof(McCoef<double>))) != MMC_OK) return bail(st);
  if ((st = alloc((void**)&h->ecoef, sizeof(EnCoef))) != MMC_OK) return bail(st);
  if ((st = alloc((void**)&h->partials, (size_t)h->npartials * NQ * sizeof(double))) != MMC_OK) return bail(st);
  if ((st = alloc((void**)&h->red, NQ * sizeof(double))) != MMC_OK) return bail(st);
  if ((st = alloc((void**)&h->acc, sizeof(unsigned long long))) != MMC_OK) return bail(st);
  if ((st = alloc((void**)&h->ctr, sizeof(SweepCounters))) != MMC_OK) return bail(st);
  if ((st = alloc((void**)&h->stage64, 3 * g.n * sizeof(double))) != MMC_OK) return bail(st);
  if ((st = alloc((void**)&h->field64, 3 * g.n * sizeof(double))) != MMC_OK) return bail(st);
  for (auto& e : h->ev)
    if (cudaEventCreate(&e) != cudaSuccess) return bail(fail(MMC_ERR_CUDA, "event creation failed"));
  if (cudaMallocHost(&h->red_host, NQ * sizeof(double)) != cudaSuccess)
    return bail(fail(MMC_ERR_OOM, "pinned allocation failed"));
  if (cudaMemset(h->acc, 0, sizeof(unsigned long long)) != cudaSuccess ||
      cudaMemset(h->h, 0, 3 * g.n * h->tsize) != cudaSuccess ||
      (h->spec && cudaMemset(h->spec, 0, 3 * g.nspec * csize) != cudaSuccess) ||
      (h->khat && cudaMemset(h->khat, 0, 6 * g.nspec * csize) != cudaSuccess))
    return bail(fail(MMC_ERR_CUDA, "memset failed"));
  if ((st = setup_engine(h, nsm)) != MMC_OK) return bail(st);
  // initial magnetisation (src/main.cu:289-333)
  if (cfg->use_random_init) {
    cudaError_t e = h->prec == 32 ? launch_init<float>(g, (uint64_t)h->seed, (float*)h->m, h->st)
                                  : launch_init<double>(g, (uint64_t)h->seed, (double*)h->m, h->st);
    if (e != cudaSuccess || cudaStreamSynchronize(h->st) != cudaSuccess)
      return bail(fail(MMC_ERR_CUDA, "init kernel failed"));
  } else if (cfg->ovf_filename[0]) {
    std::vector<double> mm(3 * g.n);
    if ((st = ovf_read(cfg->ovf_filename, g.nx, g.ny, g.nz, cfg->dx, cfg->dy, cfg->dz, mm.data(), mm.data() + g.n,
                       mm.data() + 2 * g.n)) != MMC_OK)
      return bail(st);
    if ((st = unit_vectors(mm.data(), g.n, cfg->ovf_filename)) != MMC_OK) return bail(st);
    if ((st = set_m_impl(h, mm.data(), mm.data() + g.n, mm.data() + 2 * g.n)) != MMC_OK) return bail(st);
  } else {
    std::vector<double> mm(3 * g.n, 0.0);
    for (long long i = 0; i < g.n; ++i) mm[2 * g.n + i] = 1.0;
    if ((st = set_m_impl(h, mm.data(), mm.data() + g.n, mm.data() + 2 * g.n)) != MMC_OK) return bail(st);
  }
  clear_error();
  *out = h;
  return MMC_OK;
}

bool has_ext(const std::string& f, const char* e) {
  size_t n = std::strlen(e);
  if (f.size() < n) return false;
  std::string t = f.substr(f.size() - n);
  for (auto& ch : t) ch = (char)std::tolower((unsigned char)ch);
  return t == e;
}

// src/main.cu:193-231: create the output folder, or empty it of images and OVF files.
int prepare_output_dir(const std::string& dir) {
  if (!dir_exists(dir)) {
    std::string acc;
    for (size_t i = 0; i <= dir.size(); ++i) {
      if (i == dir.size() || dir[i] == '/') {
        acc = dir.substr(0, i);
        if (!acc.empty() && !dir_exists(acc)) mkdir(acc.c_str(), 0755);
      }
    }
    if (!dir_exists(dir)) return fail(MMC_ERR_IO, "cannot create output folder: " + dir);
    return MMC_OK;
  }
  DIR* d = opendir(dir.c_str());
  if (!d) return fail(MMC_ERR_IO, "cannot open output folder: " + dir);
  while (struct dirent* e = readdir(d)) {
    std::string f = e->d_name;
    if (has_ext(f, ".ovf") || has_ext(f, ".png") || has_ext(f, ".jpg") || has_ext(f, ".jpeg"))
      std::remove(join(dir, f).c_str());
  }
  closedir(d);
  return MMC_OK;
}

int snapshot(mmc_handle* h, const std::string& dir, long long count, double T, long long sweep) {
  const long long n = h->g.n;
  std::vector<double> mm(3 * n);
  TRY(get_m_impl(h, mm.data(), mm.data() + n, mm.data() + 2 * n));
  char name[256];
  std::snprintf(name, sizeof name, "%06lld_%.2fK_%lld.ovf", count, T, sweep);
  return ovf_write(join(dir, name), h->g.nx, h->g.ny, h->g.nz, h->cfg.dx, h->cfg.dy, h->cfg.dz, mm.data(),
                   mm.data() + n, mm.data() + 2 * n, h->cfg.ovf_format, "m");
}

// One term of the effective field (enum mmc_term) in A/m, into host arrays.
int field_to_host(mmc_handle* h, int term, double* out3) {
  HCoef k = make_h_coef(h);
  cudaError_t e = h->prec == 32 ? launch_field<float>(h->g, k, term, (const float*)h->m, (const float*)h->h,
                                                      h->field64, h->st)
                                : launch_field<double>(h->g, k, term, (const double*)h->m, (const double*)h->h,
                                                       h->field64, h->st);
  CU(e);
  CU(cudaMemcpyAsync(out3, h->field64, 3 * h->g.n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  return sync_check(h);
}

// The per-term dumps of the reference's DEBUG_H_FIELD build (src/main.cu:965-1086),
// written over the same files at every energy output: B_demag, B_anis, B_exch,
// B_dmi and B_effective (mu0 H in T; B_effective includes B_ext) and
// E_density (the energy density in J/m^3, in all three columns as there).
// The demag field is the one the energy evaluation just computed for the
// current state.  The reference's B_exch kernel body is not published; here
// exchange and interfacial DMI are written apart.  Its mc_E_density (the
// Metropolis kernel's per-cell energy, also unpublished) is not written.
// E_density splits the energy by cells as
//   e_i = -(mu0 Ms / 2) m_i.(H_ex + H_dm + H_an + H_d)_i - mu0 Ms m_i.H_zeeman,
// whose sum times the cell volume is the total energy.
int dump_fields(mmc_handle* h, const std::string& dir) {
  const mmc_config& c = h->cfg;
  const long long n = h->g.n;
  const double mu0 = 4e-7 * pi_of(&c);
  std::vector<double> m(3 * n), f(3 * n), e(3 * n, 0.0);
  TRY(get_m_impl(h, m.data(), m.data() + n, m.data() + 2 * n));
  struct Dump {
    int term;
    const char* name;  // file stem, also the OVF title; none for the Zeeman term
  };
  const Dump dumps[] = {{MMC_TERM_DEMAG, "B_demag"}, {MMC_TERM_ANISOTROPY, "B_anis"},
                        {MMC_TERM_EXCHANGE, "B_exch"}, {MMC_TERM_DMI, "B_dmi"},
                        {MMC_TERM_ZEEMAN, nullptr}, {MMC_TERM_TOTAL, "B_effective"}};
  for (const Dump& d : dumps) {
    TRY(field_to_host(h, d.term, f.data()));
    if (d.term != MMC_TERM_TOTAL) {
      const double w = d.term == MMC_TERM_ZEEMAN ? -mu0 * c.ms : -0.5 * mu0 * c.ms;
      for (long long i = 0; i < n; ++i)
        e[i] += w * (m[i] * f[i] + m[n + i] * f[n + i] + m[2 * n + i] * f[2 * n + i]);
    }
    if (!d.name) continue;
    for (auto& v : f) v *= mu0;
    TRY(ovf_write(join(dir, std::string(d.name) + ".ovf"), h->g.nx, h->g.ny, h->g.nz, c.dx, c.dy, c.dz, f.data(),
                  f.data() + n, f.data() + 2 * n, c.ovf_format, d.name, "B_x B_y B_z", "T T T"));
  }
  for (long long i = 0; i < n; ++i) e[n + i] = e[2 * n + i] = e[i];
  return ovf_write(join(dir, "E_density.ovf"), h->g.nx, h->g.ny, h->g.nz, c.dx, c.dy, c.dz, e.data(),
                   e.data() + n, e.data() + 2 * n, c.ovf_format, "E_density", "E E E", "J/m3 J/m3 J/m3");
}

// The temperature-stage loop (src/main.cu:801-1139).  T is stepped in the
// working precision as the reference's FLOAT_ Temperature is.
template <typename R>
int anneal_loop(mmc_handle* h, const std::string& dir, int verbose) {
  const mmc_config& c = h->cfg;
  const std::string efile = join(dir, "energy.txt");
  {
    FILE* fp = std::fopen(efile.c_str(), "w");
    if (!fp) return fail(MMC_ERR_IO, "cannot create " + efile);
    std::fclose(fp);
  }
  R T = (R)c.Temperature_start;
  const R Tend = (R)c.Temperature_end, Tstep = (R)c.Temperature_step;
  long long out_count = 0, stage = 0;
  auto t0 = std::chrono::steady_clock::now();
  while (T > Tend) {
    if (verbose) std::printf("\n\nTemperature: %.2f K\n", (double)T);
    long long s = 0;
    while (s < c.circle_per_stage) {
      if (h->stop.load()) return fail(MMC_ERR_INTERRUPTED, "stop requested");
      if (s % c.terminal_output_period == 0 && verbose) {
        double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (s == 0) {
          t0 = std::chrono::steady_clock::now();
          std::printf("Stage: %lld \n", s);
        } else {
          std::printf("Stage: %lld, elapsed time: %f s, speed: %f stages/s\n", s, el, (double)s / el);
        }
      }
      if (s % c.ms_output_period == 0) {
        TRY(snapshot(h, dir, out_count, (double)T, s));
        ++out_count;
      }
      if (s % c.energy_output_period == 0) {
        mmc_observables o;
        TRY(energy_impl(h, &o));
        if (verbose) std::printf("\nEnergy:  %g\n", o.e_total);
        FILE* fp = std::fopen(efile.c_str(), "a");
        if (!fp) return fail(MMC_ERR_IO, "cannot append to " + efile);
        std::fprintf(fp, "%f %lld %g\n", (double)T, s, o.e_total);
        std::fclose(fp);
        if (c.debug_h_field) TRY(dump_fields(h, dir));
      }
      long long next = c.circle_per_stage;
      const long long per[3] = {c.terminal_output_period, c.ms_output_period, c.energy_output_period};
      for (long long p : per) next = std::min(next, (s / p + 1) * p);
      TRY(run_sweeps_impl(h, (double)T, stage, s, next - s));
      s = next;
    }
    T = c.Temperature_use_exp ? (R)(T * Tstep) : (R)(T - Tstep);
    ++stage;
  }
  if (verbose) std::printf("~~~~~~~~~~~~~~END~~~~~~~~~~~~~~~~~~~~~~~~~ \n");
  return MMC_OK;
}

}  // namespace


// =================================================================== batches
// nrep replicas of one geometry advanced together: every pass kernel runs over
// all replicas (grid.z = replica), which fills the GPU where one lattice only
// fills a corner of it.  Replicas may differ in material, field, seed and
// temperature; the tensor spectrum is shared.  Optional parallel-tempering
// ladders swap temperatures on the device every `swap_interval` sweeps.
constexpr int CTR_SLOTS = 32;

struct mmc_batch {
  mmc_handle* base = nullptr;  // geometry, plans, tensor (replica 0's config)
  int R = 0;
  DemagTuning tun{};
  int streams = 1;               // > 1: the batch's replicas split in that many parts on as many streams
  cudaStream_t sts[3] = {nullptr, nullptr, nullptr};  // the extra streams, created on first use
  cudaEvent_t fork = nullptr, joins[3] = {nullptr, nullptr, nullptr};
  int rows_band = 0;  // > 0: film sweeps run as row kernel + column pass
  std::vector<int> row_bands;  // bands the row kernel can run with on this device
  std::vector<mmc_config> cfgs;
  std::vector<long long> seeds;
  std::vector<double> T;
  McParams* params = nullptr;  // device, R
  void* m = nullptr;
  void* h = nullptr;
  void* spec = nullptr;
  void* m2 = nullptr;     // row kernel path: second copies of m and of the spectrum
  void* spec2 = nullptr;
  void* coef = nullptr;
  EnCoef* ecoef = nullptr;
  double* partials = nullptr;
  double* red = nullptr;
  double* red_host = nullptr;
  unsigned long long* acc = nullptr;
  // CTR_SLOTS counters, slot q = (stage, sweep + q): sweep q of a captured
  // graph reads slot q, and one advance per graph moves them all on
  SweepCounters* ctr = nullptr;
  SweepCounters ctr_host[CTR_SLOTS];
  // parallel tempering
  int interval = 0;
  PtDevice pt{};
  int* d_replica_at = nullptr;
  double* d_temps = nullptr;
  double* d_replica_T = nullptr;
  unsigned int* d_round = nullptr;
  unsigned long long* d_counts = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int graph_len = 0;
  bool graph_pt = false;
  // tempering: the graph of one swap interval whose first sweep also makes the
  // previous interval's swap (batch_sweep_lead)
  cudaGraphExec_t gexec_lead = nullptr;
  int lead_len = 0;
  std::vector<unsigned long long> acc_base;
  unsigned long long proposed = 0;
  double last_ms = 0;
  std::atomic<int> stop{0};
};

namespace {

bool same_geometry(const mmc_config& a, const mmc_config& b) {
  return a.nx == b.nx && a.ny == b.ny && a.nz == b.nz && a.dx == b.dx && a.dy == b.dy && a.dz == b.dz &&
         a.pbc_x == b.pbc_x && a.pbc_y == b.pbc_y && a.pbc_z == b.pbc_z && a.precision == b.precision &&
         a.cal_demag_flag == b.cal_demag_flag && a.use_reference_pi == b.use_reference_pi;
}

void batch_free(mmc_batch* b) {
  if (!b) return;
  if (b->base) cudaSetDevice(b->base->device);
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  if (b->gexec_lead) cudaGraphExecDestroy(b->gexec_lead);
  if (b->fork) cudaEventDestroy(b->fork);
  for (int k = 0; k < 3; ++k) {
    if (b->joins[k]) cudaEventDestroy(b->joins[k]);
    if (b->sts[k]) cudaStreamDestroy(b->sts[k]);
  }
  void* bufs[] = {b->params,   b->m,           b->h,          b->spec,        b->coef,   b->ecoef,
                  b->partials, b->red,         b->acc,        b->ctr,         b->d_replica_at,
                  b->d_temps,  b->d_replica_T, b->d_round,    b->d_counts,    b->m2,     b->spec2};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (b->red_host) cudaFreeHost(b->red_host);
  if (b->base) destroy_impl(b->base);
  delete b;
}

template <typename T>
int batch_upload_coefs(mmc_batch* b) {
  std::vector<McCoef<T>> c(b->R);
  std::vector<McParams> p(b->R);
  for (int r = 0; r < b->R; ++r) {
    p[r] = make_mc_params(b->cfgs[r], b->base->k0, b->seeds[r]);
    c[r] = mc_coef_from<T>(p[r], b->T[r]);
  }
  CU(cudaMemcpy(b->params, p.data(), b->R * sizeof(McParams), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(b->coef, c.data(), b->R * sizeof(McCoef<T>), cudaMemcpyHostToDevice));
  return MMC_OK;
}

// The demag field of every replica from m (default: the batch's m).
cudaError_t batch_demag(mmc_batch* b, cudaEvent_t* ev = nullptr, const void* m = nullptr) {
  mmc_handle* h = b->base;
  if (!m) m = b->m;
  if (h->prec == 32)
    return launch_demag<float>(h->g, h->px.p, h->py.p, h->pz.p, b->tun, (const float*)m, (float*)b->h, b->spec,
                               h->khat, h->st, b->R, ev);
  return launch_demag<double>(h->g, h->px.p, h->py.p, h->pz.p, b->tun, (const double*)m, (double*)b->h, b->spec,
                              h->khat, h->st, b->R, ev);
}

// The strip form (both colours in one launch) reads m from one copy and
// writes the other: sweep q of a run reads m on even q and m2 on odd q.
bool batch_strip(const mmc_batch* b) {
  return b->rows_band == 0 && b->tun.mc_form == MC_FORM_STRIP && mc_strip_eligible(b->base->g);
}
int batch_alloc_m2(mmc_batch* b) {
  const mmc_handle* h = b->base;
  if (!b->m2) CU(cudaMalloc(&b->m2, (size_t)b->R * 3 * h->g.n * h->tsize));
  return MMC_OK;
}
// After an odd number of strip-form sweeps the state sits in m2: move it back.
cudaError_t batch_strip_settle(mmc_batch* b) {
  mmc_handle* h = b->base;
  return cudaMemcpyAsync(b->m, b->m2, (size_t)b->R * 3 * h->g.n * h->tsize, cudaMemcpyDeviceToDevice, h->st);
}

// The second copies of m and of the spectrum that the row kernel path needs.
int batch_alloc_rows(mmc_batch* b) {
  const mmc_handle* h = b->base;
  const size_t ts = h->tsize;
  if (!b->m2) CU(cudaMalloc(&b->m2, (size_t)b->R * 3 * h->g.n * ts));
  if (!b->spec2) CU(cudaMalloc(&b->spec2, (size_t)b->R * 3 * h->g.nspec * 2 * ts));
  return MMC_OK;
}

// Film sweep as two launches: the row kernel (m, spec) -> (m2, spec2) on even
// parity, back on odd, then the column pass on the written spectrum.  Requires
// the read spectrum to hold K^.M^/N of the read m (the previous sweep's column
// pass, or batch_demag).  ev (optional): [0] before the row kernel, [1] before
// the column pass, [2] after it.
cudaError_t batch_sweep_rows(mmc_batch* b, int parity, cudaEvent_t* ev, int slot) {
  mmc_handle* h = b->base;
  void* mi = parity ? b->m2 : b->m;
  void* mo = parity ? b->m : b->m2;
  void* si = parity ? b->spec2 : b->spec;
  void* so = parity ? b->spec : b->spec2;
  cudaError_t e;
  if (ev && (e = cudaEventRecord(ev[0], h->st)) != cudaSuccess) return e;
  e = h->prec == 32 ? launch_rows<float>(h->g, h->px.p, (const McCoef<float>*)b->coef, (const float*)mi, (float*)mo,
                                         (float*)b->h, si, so, b->acc, b->ctr + slot, b->rows_band, b->R, false, true, h->st)
                    : launch_rows<double>(h->g, h->px.p, (const McCoef<double>*)b->coef, (const double*)mi,
                                          (double*)mo, (double*)b->h, si, so, b->acc, b->ctr + slot, b->rows_band, b->R,
                                          false, true, h->st);
  if (e != cudaSuccess) return e;
  if (ev && (e = cudaEventRecord(ev[1], h->st)) != cudaSuccess) return e;
  e = h->prec == 32 ? launch_col_pass_2d<float>(h->g, h->py.p, b->tun, so, h->khat, h->st, b->R)
                    : launch_col_pass_2d<double>(h->g, h->py.p, b->tun, so, h->khat, h->st, b->R);
  if (e != cudaSuccess) return e;
  if (ev && (e = cudaEventRecord(ev[2], h->st)) != cudaSuccess) return e;
  return cudaSuccess;
}

// After an odd number of row-kernel sweeps the state sits in the second
// copies; move it back so m and spec are current again.
cudaError_t batch_rows_settle(mmc_batch* b) {
  mmc_handle* h = b->base;
  cudaError_t e = cudaMemcpyAsync(b->m, b->m2, (size_t)b->R * 3 * h->g.n * h->tsize, cudaMemcpyDeviceToDevice, h->st);
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(b->spec, b->spec2, (size_t)b->R * 3 * h->g.nspec * 2 * h->tsize, cudaMemcpyDeviceToDevice,
                         h->st);
}

// The extra streams and their fork/join events.
int batch_alloc_streams(mmc_batch* b) {
  if (!b->fork) CU(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
  for (int k = 0; k < 3; ++k) {
    if (!b->sts[k]) CU(cudaStreamCreateWithFlags(&b->sts[k], cudaStreamNonBlocking));
    if (!b->joins[k]) CU(cudaEventCreateWithFlags(&b->joins[k], cudaEventDisableTiming));
  }
  return MMC_OK;
}

// One sweep of replicas [r0, r0 + nr) on stream st (parity: see batch_strip).
template <typename T>
cudaError_t batch_sweep_part(mmc_batch* b, int r0, int nr, cudaStream_t st, int slot, int parity) {
  mmc_handle* h = b->base;
  const long long ms = 3 * h->g.n, ss = 3 * h->g.nspec;
  const bool strip = batch_strip(b);
  T* m = (T*)(strip && parity ? b->m2 : b->m) + r0 * ms;
  T* hh = (T*)b->h + r0 * ms;
  cudaError_t e = cudaSuccess;
  if (h->cfg.cal_demag_flag)
    e = launch_demag<T>(h->g, h->px.p, h->py.p, h->pz.p, b->tun, m, hh,
                        (char*)b->spec + (size_t)r0 * ss * 2 * sizeof(T), h->khat, st, nr);
  if (e != cudaSuccess) return e;
  if (strip) {
    T* mo = (T*)(parity ? b->m : b->m2) + r0 * ms;
    return launch_mc_strip<T>(h->g, (const McCoef<T>*)b->coef + r0, m, mo, hh, b->ctr + slot, b->acc + r0, st, nr);
  }
  return launch_mc<T>(h->g, (const McCoef<T>*)b->coef + r0, m, hh, b->ctr + slot, -1, b->acc + r0, st, nr,
                      b->tun.mc_form);
}

// One sweep reading counter slot `slot` (the caller advances the counters);
// parity: see batch_strip.
cudaError_t batch_sweep(mmc_batch* b, cudaEvent_t* ev, int slot, int parity) {
  mmc_handle* h = b->base;
  cudaError_t e;
  const int parts = std::min(b->streams, b->R);
  // replica parts on their own streams while a graph is captured (as parallel
  // branches, kernels of different kinds overlap on the SMs); launched
  // directly, the extra launches and events cost more than they give, and
  // every launch shape gives the same results, so direct sweeps use one stream
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (parts > 1 && (e = cudaStreamIsCapturing(h->st, &cap)) != cudaSuccess) return e;
  if (parts > 1 && !ev && b->sts[0] && cap == cudaStreamCaptureStatusActive) {
    // part 0 stays on the batch's stream
    if ((e = cudaEventRecord(b->fork, h->st)) != cudaSuccess) return e;
    for (int k = 1; k < parts; ++k)
      if ((e = cudaStreamWaitEvent(b->sts[k - 1], b->fork, 0)) != cudaSuccess) return e;
    for (int k = parts - 1; k >= 0; --k) {
      const int r0 = (int)((long long)b->R * k / parts), r1 = (int)((long long)b->R * (k + 1) / parts);
      cudaStream_t st = k == 0 ? h->st : b->sts[k - 1];
      e = h->prec == 32 ? batch_sweep_part<float>(b, r0, r1 - r0, st, slot, parity)
                        : batch_sweep_part<double>(b, r0, r1 - r0, st, slot, parity);
      if (e != cudaSuccess) return e;
    }
    for (int k = 1; k < parts; ++k) {
      if ((e = cudaEventRecord(b->joins[k - 1], b->sts[k - 1])) != cudaSuccess) return e;
      if ((e = cudaStreamWaitEvent(h->st, b->joins[k - 1], 0)) != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  const bool strip = batch_strip(b);
  void* mi = strip && parity ? b->m2 : b->m;
  void* mo = parity ? b->m : b->m2;
  if (h->cfg.cal_demag_flag && (e = batch_demag(b, ev, mi)) != cudaSuccess) return e;
  if (strip)
    e = h->prec == 32 ? launch_mc_strip<float>(h->g, (const McCoef<float>*)b->coef, (const float*)mi, (float*)mo,
                                               (const float*)b->h, b->ctr + slot, b->acc, h->st, b->R)
                      : launch_mc_strip<double>(h->g, (const McCoef<double>*)b->coef, (const double*)mi, (double*)mo,
                                                (const double*)b->h, b->ctr + slot, b->acc, h->st, b->R);
  else
    e = h->prec == 32 ? launch_mc<float>(h->g, (const McCoef<float>*)b->coef, (float*)b->m, (const float*)b->h,
                                         b->ctr + slot, -1, b->acc, h->st, b->R, b->tun.mc_form)
                      : launch_mc<double>(h->g, (const McCoef<double>*)b->coef, (double*)b->m, (const double*)b->h,
                                          b->ctr + slot, -1, b->acc, h->st, b->R, b->tun.mc_form);
  if (e != cudaSuccess) return e;
  if (ev && (e = cudaEventRecord(ev[4], h->st)) != cudaSuccess) return e;
  return cudaSuccess;
}

// k sweeps; on the row kernel path they alternate between the two copies and
// end in m and spec.
// Sweep q reads counter slot q mod CTR_SLOTS; the counters advance after
// every CTR_SLOTS sweeps and after the last one (one small launch per graph
// of 32 sweeps instead of one per sweep).
cudaError_t batch_swap(mmc_batch* b);
cudaError_t batch_energy_kernels(mmc_batch* b, bool swap = false, bool with_demag = true);
// The first sweep of a swap interval that also makes the previous interval's
// swap: the demag field of m (which the sweep needs anyway) gives the
// energies, the swap pass updates the temperatures, then the Metropolis
// launches run -- one demag evaluation where a separate swap pass would need
// its own.  The same energies, swaps and decisions as a swap pass followed by
// a sweep.
cudaError_t batch_sweep_lead(mmc_batch* b, int slot) {
  mmc_handle* h = b->base;
  cudaError_t e;
  if (h->cfg.cal_demag_flag && (e = batch_demag(b)) != cudaSuccess) return e;
  if ((e = batch_energy_kernels(b, true, false)) != cudaSuccess) return e;
  if ((e = batch_swap(b)) != cudaSuccess) return e;
  if (batch_strip(b))
    return h->prec == 32 ? launch_mc_strip<float>(h->g, (const McCoef<float>*)b->coef, (const float*)b->m,
                                                  (float*)b->m2, (const float*)b->h, b->ctr + slot, b->acc, h->st, b->R)
                         : launch_mc_strip<double>(h->g, (const McCoef<double>*)b->coef, (const double*)b->m,
                                                   (double*)b->m2, (const double*)b->h, b->ctr + slot, b->acc, h->st,
                                                   b->R);
  return h->prec == 32 ? launch_mc<float>(h->g, (const McCoef<float>*)b->coef, (float*)b->m, (const float*)b->h,
                                          b->ctr + slot, -1, b->acc, h->st, b->R, b->tun.mc_form)
                       : launch_mc<double>(h->g, (const McCoef<double>*)b->coef, (double*)b->m, (const double*)b->h,
                                           b->ctr + slot, -1, b->acc, h->st, b->R, b->tun.mc_form);
}

// lead_swap: the first sweep makes the pending swap (batch_sweep_lead; the
// pass kernels path only).
cudaError_t batch_sweeps(mmc_batch* b, long long k, bool lead_swap = false) {
  cudaError_t e = cudaSuccess;
  for (long long q = 0; q < k && e == cudaSuccess; ++q) {
    const int slot = (int)(q % CTR_SLOTS);
    e = (q == 0 && lead_swap) ? batch_sweep_lead(b, slot)
        : b->rows_band > 0    ? batch_sweep_rows(b, (int)(q & 1), nullptr, slot)
                              : batch_sweep(b, nullptr, slot, (int)(q & 1));
    if (e == cudaSuccess && (slot == CTR_SLOTS - 1 || q == k - 1))
      e = launch_advance(b->ctr, (uint32_t)(slot + 1), b->base->st, CTR_SLOTS);
  }
  if (e == cudaSuccess && b->rows_band > 0 && (k & 1)) e = batch_rows_settle(b);
  if (e == cudaSuccess && batch_strip(b) && (k & 1)) e = batch_strip_settle(b);
  return e;
}

// Sets the counter slots to (stage, sweep0 + q).
cudaError_t batch_set_counters(mmc_batch* b, long long stage, long long sweep0) {
  for (int q = 0; q < CTR_SLOTS; ++q) b->ctr_host[q] = SweepCounters{(uint32_t)stage, (uint32_t)(sweep0 + q)};
  return cudaMemcpyAsync(b->ctr, b->ctr_host, sizeof b->ctr_host, cudaMemcpyHostToDevice, b->base->st);
}

// Energies (and <m> and the topological charge) of every replica into b->red;
// swap = true: the energies a tempering swap needs (launch_energy, with_q = -1).
// with_demag = false: b->h already holds the demag field of b->m.
cudaError_t batch_energy_kernels(mmc_batch* b, bool swap, bool with_demag) {
  const int with_q = swap ? -1 : 1;
  mmc_handle* h = b->base;
  cudaError_t e;
  if (with_demag && h->cfg.cal_demag_flag && (e = batch_demag(b)) != cudaSuccess) return e;
  const bool dm = h->cfg.cal_demag_flag != 0;
  return h->prec == 32 ? launch_energy<float>(h->g, b->ecoef, (const float*)b->m, dm ? (const float*)b->h : nullptr,
                                              b->partials, h->npartials, b->red, h->st, b->R, with_q)
                       : launch_energy<double>(h->g, b->ecoef, (const double*)b->m,
                                               dm ? (const double*)b->h : nullptr, b->partials, h->npartials,
                                               b->red, h->st, b->R, with_q);
}

cudaError_t batch_swap(mmc_batch* b) {
  mmc_handle* h = b->base;
  return h->prec == 32 ? launch_pt_swap<float>(b->pt, b->params, (McCoef<float>*)b->coef, b->red, h->st)
                       : launch_pt_swap<double>(b->pt, b->params, (McCoef<double>*)b->coef, b->red, h->st);
}

// A graph of `len` sweeps, followed (pt) by an energy evaluation and a swap pass.
// The graph of one swap interval of `len` sweeps whose first sweep makes the
// pending swap (batch_sweep_lead).
int batch_graph_lead(mmc_batch* b, int len) {
  if (b->gexec_lead && b->lead_len == len) return MMC_OK;
  if (b->gexec_lead) cudaGraphExecDestroy(b->gexec_lead);
  b->gexec_lead = nullptr;
  mmc_handle* h = b->base;
  cudaGraph_t graph;
  CU(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = batch_sweeps(b, len, true);
  cudaError_t e2 = cudaStreamEndCapture(h->st, &graph);
  if (e != cudaSuccess || e2 != cudaSuccess) cudaGetLastError();
  if (e != cudaSuccess) return fail(MMC_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(e));
  if (e2 != cudaSuccess) return fail(MMC_ERR_CUDA, std::string("batch capture end: ") + cudaGetErrorString(e2));
  e = cudaGraphInstantiate(&b->gexec_lead, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return fail(MMC_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(e));
  b->lead_len = len;
  return MMC_OK;
}

// Drops the captured graphs (launch shape, ladders or the state they bind changed).
void batch_drop_graphs(mmc_batch* b) {
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  b->graph_len = 0;
  if (b->gexec_lead) cudaGraphExecDestroy(b->gexec_lead);
  b->gexec_lead = nullptr;
  b->lead_len = 0;
}

int batch_graph(mmc_batch* b, int len, bool pt) {
  if (b->gexec && b->graph_len == len && b->graph_pt == pt) return MMC_OK;
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  mmc_handle* h = b->base;
  cudaGraph_t graph;
  CU(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  e = batch_sweeps(b, len);
  if (pt && e == cudaSuccess) e = batch_energy_kernels(b, true);  // the swap reads the energies only
  if (pt && e == cudaSuccess) e = batch_swap(b);
  cudaError_t e2 = cudaStreamEndCapture(h->st, &graph);
  if (e != cudaSuccess || e2 != cudaSuccess) cudaGetLastError();
  if (e != cudaSuccess) return fail(MMC_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(e));
  if (e2 != cudaSuccess) return fail(MMC_ERR_CUDA, std::string("batch capture end: ") + cudaGetErrorString(e2));
  e = cudaGraphInstantiate(&b->gexec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return fail(MMC_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(e));
  b->graph_len = len;
  b->graph_pt = pt;
  return MMC_OK;
}

int batch_sync_temperatures(mmc_batch* b) {
  if (b->interval > 0) CU(cudaMemcpy(b->T.data(), b->d_replica_T, b->R * sizeof(double), cudaMemcpyDeviceToHost));
  return MMC_OK;
}

// A run of nsweeps sweeps enqueued in pieces (a graph of 32 sweeps, or of one
// swap interval followed by the swap pass), so that the pieces of several
// batches can be interleaved on their own streams (mmc_farm_run_sweeps).
struct BatchRun {
  long long stage = 0, sweep0 = 0, nsweeps = 0, done = 0;
  long long pieces = 0;
  bool swap_pending = false;  // a swap interval ended; its swap not yet made
};
constexpr int BATCH_GRAPH_SWEEPS = 32;

int batch_run_begin(mmc_batch* b, BatchRun& r, long long stage, long long sweep0, long long nsweeps) {
  mmc_handle* h = b->base;
  TRY(ensure_demag(h));
  TRY(batch_sync_temperatures(b));
  TRY(h->prec == 32 ? batch_upload_coefs<float>(b) : batch_upload_coefs<double>(b));
  CU(batch_set_counters(b, stage, sweep0));
  CU(cudaEventRecord(h->ev[0], h->st));
  if (b->rows_band > 0) CU(batch_demag(b));  // the row kernel starts from the spectrum of m
  r = BatchRun{stage, sweep0, nsweeps, 0, 0};
  if (b->interval == 0 && nsweeps >= BATCH_GRAPH_SWEEPS) TRY(batch_graph(b, BATCH_GRAPH_SWEEPS, false));
  return MMC_OK;
}

int batch_run_piece(mmc_batch* b, BatchRun& r, bool* finished) {
  mmc_handle* h = b->base;
  const int I = b->interval;
  if (r.done < r.nsweeps) {
    if (I > 0) {
      // sweeps up to the next multiple of the swap interval, after which a
      // swap is due; it is made by the next interval's first sweep
      // (batch_sweep_lead, one demag evaluation less), or by a swap pass
      // before direct sweeps or at the end of the run
      const long long s = r.sweep0 + r.done;
      const long long to_boundary = I - (s % I);
      const bool lead_ok = b->rows_band == 0;
      if (to_boundary <= r.nsweeps - r.done && to_boundary == I && (!r.swap_pending || lead_ok)) {
        if (r.swap_pending) {
          TRY(batch_graph_lead(b, I));
          CU(cudaGraphLaunch(b->gexec_lead, h->st));
        } else {
          TRY(batch_graph(b, I, false));
          CU(cudaGraphLaunch(b->gexec, h->st));
        }
        r.done += I;
        r.swap_pending = true;
      } else {
        if (r.swap_pending) {
          CU(batch_energy_kernels(b, true));
          CU(batch_swap(b));
          r.swap_pending = false;
        }
        const long long k = std::min(to_boundary, r.nsweeps - r.done);
        CU(batch_sweeps(b, k));
        r.done += k;
        r.swap_pending = k == to_boundary;
      }
    } else if (r.nsweeps - r.done >= BATCH_GRAPH_SWEEPS) {
      CU(cudaGraphLaunch(b->gexec, h->st));
      r.done += BATCH_GRAPH_SWEEPS;
    } else {
      CU(batch_sweeps(b, r.nsweeps - r.done));
      r.done = r.nsweeps;
    }
    ++r.pieces;
  }
  *finished = r.done >= r.nsweeps;
  return MMC_OK;
}

int batch_run_end(mmc_batch* b, BatchRun& r) {
  mmc_handle* h = b->base;
  if (r.swap_pending) {
    CU(batch_energy_kernels(b, true));
    CU(batch_swap(b));
    r.swap_pending = false;
  }
  CU(cudaEventRecord(h->ev[1], h->st));
  CU(cudaStreamSynchronize(h->st));
  if (b->tun.mc_form == MC_FORM_PIPE && mc_pipe_error_take())
    return fail(MMC_ERR_TIMEOUT, "a pipelined Metropolis buffer wait ran out of its time limit");
  float ms = 0;
  CU(cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]));
  b->last_ms = ms;
  b->proposed += (unsigned long long)r.nsweeps * (unsigned long long)h->g.n;
  return batch_sync_temperatures(b);
}

int batch_run(mmc_batch* b, long long stage, long long sweep0, long long nsweeps) {
  BatchRun r;
  TRY(batch_run_begin(b, r, stage, sweep0, nsweeps));
  for (bool fin = false; !fin;) {
    TRY(batch_run_piece(b, r, &fin));
    if (b->stop.load()) return fail(MMC_ERR_INTERRUPTED, "stop requested");
    // bound the queued work so that a stop request takes effect quickly
    if (r.pieces % 64 == 0) CU(cudaStreamSynchronize(b->base->st));
  }
  return batch_run_end(b, r);
}

// Times every launch shape the batch can run with -- the row kernel with each
// band that fits, the pass kernels with each x-pass row count and column-pass
// width -- for `sweeps` sweeps from the current state, keeps the fastest and
// puts the state back.  All shapes give bit-identical results.
int batch_autotune(mmc_batch* b, int sweeps, double* best_ms, int* ncand) {
  mmc_handle* h = b->base;
  TRY(ensure_demag(h));
  TRY(batch_sync_temperatures(b));
  TRY(h->prec == 32 ? batch_upload_coefs<float>(b) : batch_upload_coefs<double>(b));
  struct Cand {
    int rows_band;
    DemagTuning tun;
    int streams = 1;
  };
  const Geom& g = h->g;
  const size_t cs = 2 * h->tsize;
  const DemagTuning base = choose_tuning(g, h->px.p, h->py.p, h->pz.p, cs, h->nsm, b->R);
  const size_t mbytes = (size_t)b->R * 3 * g.n * h->tsize;
  void* saved = nullptr;
  CU(cudaMalloc(&saved, mbytes));
  std::vector<unsigned long long> acc0(b->R);
  cudaError_t e = cudaMemcpyAsync(saved, b->m, mbytes, cudaMemcpyDeviceToDevice, h->st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(acc0.data(), b->acc, b->R * sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  int status = MMC_OK;
  int tried = 0;
  Cand best{0, base};
  float best_t = -1;
  // times one candidate from the saved state; keeps it when it is the fastest
  auto trial = [&](const Cand& cd) {
    if (e != cudaSuccess || status != MMC_OK) return;
    if (cd.rows_band > 0 && (status = batch_alloc_rows(b)) != MMC_OK) return;
    if (cd.streams > 1 && (status = batch_alloc_streams(b)) != MMC_OK) return;
    if (cd.tun.mc_form == MC_FORM_STRIP && (status = batch_alloc_m2(b)) != MMC_OK) return;
    ++tried;
    b->rows_band = cd.rows_band;
    b->tun = cd.tun;
    b->streams = cd.streams;
    e = cudaMemcpyAsync(b->m, saved, mbytes, cudaMemcpyDeviceToDevice, h->st);
    if (e == cudaSuccess) e = batch_set_counters(b, 0, 0);
    if (e == cudaSuccess && b->rows_band > 0) e = batch_demag(b);
    // timed the way runs execute: replays of a captured graph of
    // BATCH_GRAPH_SWEEPS sweeps with this shape
    if (e == cudaSuccess) {
      batch_drop_graphs(b);
      if ((status = batch_graph(b, BATCH_GRAPH_SWEEPS, false)) != MMC_OK) return;
    }
    const int reps = std::max(1, (sweeps + BATCH_GRAPH_SWEEPS - 1) / BATCH_GRAPH_SWEEPS);
    if (e == cudaSuccess) e = cudaGraphLaunch(b->gexec, h->st);  // warm-up
    // the faster of two timed repetitions, per sweep
    float ms = -1;
    for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) {
      if (e == cudaSuccess) e = cudaEventRecord(h->ev[0], h->st);
      for (int i = 0; i < reps && e == cudaSuccess; ++i) e = cudaGraphLaunch(b->gexec, h->st);
      if (e == cudaSuccess) e = cudaEventRecord(h->ev[1], h->st);
      if (e == cudaSuccess) e = cudaEventSynchronize(h->ev[1]);
      float t = 0;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&t, h->ev[0], h->ev[1]);
      t /= (float)(reps * BATCH_GRAPH_SWEEPS);
      if (e == cudaSuccess && (ms < 0 || t < ms)) ms = t;
    }
    if (e == cudaSuccess && (best_t < 0 || ms < best_t)) {
      best = cd;
      best_t = ms;
    }
  };
  // coordinate search: the pass-kernel tiling first, then one dimension at a
  // time from the best so far; the row kernel bands are whole alternatives
  trial({0, base});
  if (h->cfg.cal_demag_flag) {
    const long long rows = (long long)g.ny * g.nz;
    for (int r : {1, 2, 4, 8, 16}) {
      if (r > rows || x_pass_smem(h->px.p, r, cs) > smem_limit()) continue;
      for (int tx : {1, 2, 4, 8}) {
        // a tile the copying form cannot hold is tried in place
        const bool fits = col_pass_smem(h->py.p, tx, cs, base.col_lean != 0) <= smem_limit();
        const bool fits_lean = col_pass_smem(h->py.p, tx, cs, true) <= smem_limit();
        if (tx > g.hx || !(fits || fits_lean)) continue;
        if (r == base.x_rows_per_cta && tx == base.col_tx) continue;
        DemagTuning t = base;
        t.x_rows_per_cta = r;
        t.col_tx = tx;
        if (!fits) t.col_lean = 1;
        t.col_threads = col_threads_for(g, h->py.p, h->pz.p, tx, t.col_tx_z);
        trial({0, t});
      }
    }
    Cand c = best;
    c.tun.fft_inline = 1 - c.tun.fft_inline;
    trial(c);
    // the other column-pass form (in place or with copies) with the full and
    // half thread count, and the half thread count of the current form
    if (h->py.p.warp_a) {
      const Cand cur = best;
      for (int flip = 0; flip < 2; ++flip)
        for (int half = 0; half < 2; ++half) {
          if (!flip && !half) continue;
          Cand d = cur;
          if (flip) d.tun.col_lean = 1 - cur.tun.col_lean;
          if (half) d.tun.col_threads = std::max(64, cur.tun.col_threads / 2);
          if (half && d.tun.col_threads == cur.tun.col_threads) continue;
          if (col_pass_smem(h->py.p, d.tun.col_tx, cs, d.tun.col_lean != 0) > smem_limit()) continue;
          trial(d);
        }
    }
  }
  // the column pass held in registers (films with y lengths 64 and 256):
  // col_lean = 2 all three components per thread, 3 one component per thread
  if (h->cfg.cal_demag_flag && g.nzp == 1 && h->py.p.warp_a == h->py.p.warp_b &&
      (h->py.p.warp_a == 8 || h->py.p.warp_a == 16)) {
    const Cand base = best;
    for (int form = 2; form <= 3; ++form) {
      Cand c = base;
      c.tun.col_lean = form;
      trial(c);
    }
  }
  {
    std::vector<int> forms;
    if (mc_strip_eligible(g) && mc_strip_smem_bytes(g, h->tsize) <= smem_limit()) forms.push_back(MC_FORM_STRIP);
    if (mc_pipe_eligible(g) && mc_pipe_smem_bytes(g, h->tsize) <= smem_limit()) forms.push_back(MC_FORM_PIPE);
    if (mc_quad_eligible(g)) forms.push_back(MC_FORM_QUAD);
    if (mc_band_eligible(g)) forms.push_back(MC_FORM_BAND);
    if (mc_tile_eligible(g)) forms.push_back(MC_FORM_TILE);
    forms.push_back(MC_FORM_SCALAR);
    const Cand pass_best = best;
    for (int f : forms)
      if (f != pass_best.tun.mc_form) {
        Cand c = pass_best;
        c.tun.mc_form = f;
        trial(c);
      }
  }
  {  // replica parts on 2, 3 or 4 streams
    const Cand one = best;
    for (int k = 2; k <= std::min(4, b->R); ++k) {
      Cand c = one;
      c.streams = k;
      trial(c);
    }
  }
  if (h->cfg.cal_demag_flag)
    for (int bd : b->row_bands) {
      Cand c = best;
      c.rows_band = bd;
      c.streams = 1;
      trial(c);
    }
  if (e == cudaSuccess && status == MMC_OK && best_t >= 0) {
    b->rows_band = best.rows_band;
    b->tun = best.tun;
    b->streams = best.streams;
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(b->m, saved, mbytes, cudaMemcpyDeviceToDevice, h->st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->acc, acc0.data(), b->R * sizeof(unsigned long long), cudaMemcpyHostToDevice, h->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  cudaFree(saved);
  batch_drop_graphs(b);
  if (status != MMC_OK) return status;
  CU(e);
  if (mc_pipe_error_take()) return fail(MMC_ERR_TIMEOUT, "a pipelined Metropolis buffer wait ran out of its time limit");
  if (best_ms) *best_ms = best_t;
  if (ncand) *ncand = tried;
  return MMC_OK;
}

int batch_create_impl(const mmc_config* cfgs, int R, int device, mmc_batch** out) {
  *out = nullptr;
  if (R < 1 || R > 65535) return fail(MMC_ERR_INVALID, "replica count must be in [1, 65535]");
  for (int r = 0; r < R; ++r) {
    TRY(config_validate(&cfgs[r]));
    if (!same_geometry(cfgs[0], cfgs[r]))
      return fail(MMC_ERR_INVALID, "batch replicas must share lattice, cell size, pbc, precision and demag flag");
  }
  mmc_batch* b = new mmc_batch();
  mmc_config c0 = cfgs[0];
  c0.sweep_engine = MMC_ENGINE_KERNELS;
  c0.use_random_init = 1;  // the base lattice's own m is unused
  int st = create_impl(&c0, device, &b->base);
  if (st != MMC_OK) {
    delete b;
    return st;
  }
  mmc_handle* h = b->base;
  b->R = R;
  b->tun = choose_tuning(h->g, h->px.p, h->py.p, h->pz.p, 2 * h->tsize, h->nsm, R);
  {
    const Geom& gg = h->g;
    const bool film = h->cfg.cal_demag_flag && gg.nz == 1 && gg.nzp == 1 && gg.ncolors == 2 &&
                      ((size_t)gg.nx * h->tsize) % 16 == 0 && ((size_t)gg.hxp * 2 * h->tsize) % 16 == 0 &&
                      h->px.p.warp_a != 32 && h->py.p.warp_a != 32;
    int optin = 48 * 1024;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
    if (film) {
      const int bands[] = {4, 2, 8, 1};
      for (int bd : bands) {
        const size_t sm = h->prec == 32 ? rows_smem_bytes<float>(gg, h->px.p, bd)
                                        : rows_smem_bytes<double>(gg, h->px.p, bd);
        if (sm > (size_t)optin || bd > 60) continue;
        int per_sm = 0;
        cudaError_t e = h->prec == 32 ? rows_prepare<float>(gg, h->px.p, bd, &per_sm)
                                      : rows_prepare<double>(gg, h->px.p, bd, &per_sm);
        if (e == cudaSuccess && per_sm >= 1) b->row_bands.push_back(bd);
      }
      cudaGetLastError();
    }
    // the row kernel path on request; the autotuner may pick it as well
    if (cfgs[0].sweep_engine == MMC_ENGINE_FUSED) {
      if (b->row_bands.empty()) {
        batch_free(b);
        return fail(MMC_ERR_UNSUPPORTED,
                    "the row-kernel batch path needs films (nz = 1) with demag, two colours, 16-byte rows and "
                    "padded sides other than 512 and 1024");
      }
      b->rows_band = b->row_bands[0];
    }
  }
  b->cfgs.assign(cfgs, cfgs + R);
  for (int r = 0; r < R; ++r) {
    b->seeds.push_back(cfgs[r].randomseed < 0 ? (long long)std::time(nullptr) + r : cfgs[r].randomseed);
    b->T.push_back(cfgs[r].Temperature_start);
  }
  b->acc_base.assign(R, 0);
  const Geom& g = h->g;
  const size_t ts = h->tsize, cs = 2 * ts;
  auto bail = [&](int s) {
    std::string msg = last_error_cstr();
    batch_free(b);
    fail(s, msg);
    return s;
  };
  auto alloc = [&](void** p, size_t bytes) -> int {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return fail(MMC_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return MMC_OK;
  };
  if ((st = alloc((void**)&b->params, R * sizeof(McParams))) != MMC_OK) return bail(st);
  if ((st = alloc(&b->m, (size_t)R * 3 * g.n * ts)) != MMC_OK) return bail(st);
  if ((st = alloc(&b->h, (size_t)R * 3 * g.n * ts)) != MMC_OK) return bail(st);
  if (h->cfg.cal_demag_flag && (st = alloc(&b->spec, (size_t)R * 3 * g.nspec * cs)) != MMC_OK) return bail(st);
  if (b->rows_band > 0 && (st = batch_alloc_rows(b)) != MMC_OK) return bail(st);
  if ((st = alloc(&b->coef, R * sizeof(McCoef<double>))) != MMC_OK) return bail(st);
  if ((st = alloc((void**)&b->ecoef, R * sizeof(EnCoef))) != MMC_OK) return bail(st);
  if ((st = alloc((void**)&b->partials, (size_t)R * h->npartials * NQ * sizeof(double))) != MMC_OK) return bail(st);
  if ((st = alloc((void**)&b->red, (size_t)R * NQ * sizeof(double))) != MMC_OK) return bail(st);
  if ((st = alloc((void**)&b->acc, R * sizeof(unsigned long long))) != MMC_OK) return bail(st);
  if ((st = alloc((void**)&b->ctr, CTR_SLOTS * sizeof(SweepCounters))) != MMC_OK) return bail(st);
  if (cudaMallocHost(&b->red_host, (size_t)R * NQ * sizeof(double)) != cudaSuccess)
    return bail(fail(MMC_ERR_OOM, "pinned allocation failed"));
  if (cudaMemset(b->acc, 0, R * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMemset(b->h, 0, (size_t)R * 3 * g.n * ts) != cudaSuccess ||
      (b->spec && cudaMemset(b->spec, 0, (size_t)R * 3 * g.nspec * cs) != cudaSuccess))
    return bail(fail(MMC_ERR_CUDA, "memset failed"));
  std::vector<EnCoef> ec(R);
  for (int r = 0; r < R; ++r) {
    mmc_handle tmp;  // only cfg is read by make_en_coef
    tmp.cfg = cfgs[r];
    ec[r] = make_en_coef(&tmp);
  }
  if (cudaMemcpy(b->ecoef, ec.data(), R * sizeof(EnCoef), cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(fail(MMC_ERR_CUDA, "coefficient upload failed"));
  // initial states: random from each replica's seed, or its OVF file
  for (int r = 0; r < R; ++r) {
    const size_t off = (size_t)r * 3 * g.n;
    if (cfgs[r].use_random_init || !cfgs[r].ovf_filename[0]) {
      cudaError_t e = h->prec == 32 ? launch_init<float>(g, (uint64_t)b->seeds[r], (float*)b->m + off, h->st)
                                    : launch_init<double>(g, (uint64_t)b->seeds[r], (double*)b->m + off, h->st);
      if (e != cudaSuccess) return bail(fail(MMC_ERR_CUDA, "init kernel failed"));
    } else {
      std::vector<double> mm(3 * g.n);
      if ((st = ovf_read(cfgs[r].ovf_filename, g.nx, g.ny, g.nz, cfgs[r].dx, cfgs[r].dy, cfgs[r].dz, mm.data(),
                         mm.data() + g.n, mm.data() + 2 * g.n)) != MMC_OK)
        return bail(st);
      if ((st = unit_vectors(mm.data(), g.n, cfgs[r].ovf_filename)) != MMC_OK) return bail(st);
      if (cudaMemcpy(h->stage64, mm.data(), 3 * g.n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(fail(MMC_ERR_CUDA, "upload failed"));
      cudaError_t e = h->prec == 32 ? launch_from_f64<float>(3 * g.n, h->stage64, (float*)b->m + off, h->st)
                                    : launch_from_f64<double>(3 * g.n, h->stage64, (double*)b->m + off, h->st);
      if (e != cudaSuccess) return bail(fail(MMC_ERR_CUDA, "conversion failed"));
    }
  }
  if (cudaStreamSynchronize(h->st) != cudaSuccess) return bail(fail(MMC_ERR_CUDA, "init failed"));
  clear_error();
  *out = b;
  return MMC_OK;
}

int batch_replica_ptr(mmc_batch* b, int r, size_t* off) {
  if (r < 0 || r >= b->R) return fail(MMC_ERR_INVALID, "replica index out of range");
  *off = (size_t)r * 3 * b->base->g.n;
  return MMC_OK;
}

}  // namespace

// =================================================================== C ABI
extern "C" {

int mmc_abi_version(void) { return MMC_ABI_VERSION; }

size_t mmc_config_size(void) { return sizeof(mmc_config); }

const char* mmc_status_string(int s) {
  switch (s) {
    case MMC_OK: return "ok";
    case MMC_ERR_INVALID: return "invalid argument";
    case MMC_ERR_CONFIG: return "configuration error";
    case MMC_ERR_IO: return "I/O error";
    case MMC_ERR_CUDA: return "CUDA error";
    case MMC_ERR_NO_DEVICE: return "no CUDA device";
    case MMC_ERR_UNSUPPORTED: return "unsupported";
    case MMC_ERR_INTERRUPTED: return "interrupted";
    case MMC_ERR_TIMEOUT: return "device wait timed out";
    case MMC_ERR_STATE: return "wrong call order";
    case MMC_ERR_OOM: return "out of device memory";
    default: return "unknown status";
  }
}

const char* mmc_last_error(void) { return last_error_cstr(); }

void mmc_config_defaults(mmc_config* cfg) {
  if (cfg) config_defaults(cfg);
}

int mmc_config_load_ini(const char* path, mmc_config* cfg) {
  if (!path || !cfg) return fail(MMC_ERR_INVALID, "null argument");
  return config_load_ini(path, cfg);
}

int mmc_config_format(const mmc_config* cfg, char* buf, size_t len) {
  if (!cfg || !buf || len == 0) return fail(MMC_ERR_INVALID, "null argument");
  std::string s = config_format(cfg);
  std::snprintf(buf, len, "%s", s.c_str());
  return MMC_OK;
}

int mmc_padded_dims(const mmc_config* cfg, int out[3]) {
  if (!cfg || !out) return fail(MMC_ERR_INVALID, "null argument");
  out[0] = cfg->pbc_x == 0 ? 2 * cfg->nx - 1 : cfg->nx;
  out[1] = cfg->pbc_y == 0 ? 2 * cfg->ny - 1 : cfg->ny;
  out[2] = cfg->pbc_z == 0 ? 2 * cfg->nz - 1 : cfg->nz;
  return MMC_OK;
}

int mmc_transform_dims(const mmc_config* cfg, int out[3]) {
  int t[3];
  TRY(mmc_padded_dims(cfg, t));
  out[0] = transform_len(t[0], cfg->pbc_x == 0);
  out[1] = transform_len(t[1], cfg->pbc_y == 0);
  out[2] = transform_len(t[2], cfg->pbc_z == 0);
  return MMC_OK;
}

int mmc_create(const mmc_config* cfg, int device, mmc_handle** out) {
  if (!cfg || !out) return fail(MMC_ERR_INVALID, "null argument");
  return create_impl(cfg, device, out);
}

void mmc_destroy(mmc_handle* h) { destroy_impl(h); }

// The handle's work moves to `stream` (NULL: its own stream); the new stream
// first waits for what the old one has enqueued.  Graphs are captured on the
// handle's stream, so the legacy and per-thread default streams are refused.
static int set_stream_impl(mmc_handle* h, void* stream) {
  cudaStream_t ns = stream ? static_cast<cudaStream_t>(stream) : h->st_own;
  if (ns == cudaStreamLegacy || ns == cudaStreamPerThread)
    return fail(MMC_ERR_INVALID, "a default stream cannot carry the handle's work (graphs are captured on it)");
  if (ns == h->st) return MMC_OK;
  TRY(set_dev(h));
  int dev = -1;
  CU(cudaStreamGetDevice(ns, &dev));
  if (dev != h->device) return fail(MMC_ERR_INVALID, "the stream belongs to another device");
  cudaEvent_t e = nullptr;
  CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  cudaError_t r = cudaEventRecord(e, h->st);
  if (r == cudaSuccess) r = cudaStreamWaitEvent(ns, e, 0);
  cudaEventDestroy(e);
  CU(r);
  h->st = ns;
  return MMC_OK;
}

int mmc_set_stream(mmc_handle* h, void* stream) {
  if (!h) return fail(MMC_ERR_INVALID, "null handle");
  return set_stream_impl(h, stream);
}

int mmc_init_random(mmc_handle* h, long long seed) {
  if (!h) return fail(MMC_ERR_INVALID, "null handle");
  TRY(set_dev(h));
  cudaError_t e = h->prec == 32 ? launch_init<float>(h->g, (uint64_t)seed, (float*)h->m, h->st)
                                : launch_init<double>(h->g, (uint64_t)seed, (double*)h->m, h->st);
  CU(e);
  return sync_check(h);
}

int mmc_set_m(mmc_handle* h, const double* mx, const double* my, const double* mz) {
  if (!h || !mx || !my || !mz) return fail(MMC_ERR_INVALID, "null argument");
  TRY(set_dev(h));
  return set_m_impl(h, mx, my, mz);
}

int mmc_get_m(mmc_handle* h, double* mx, double* my, double* mz) {
  if (!h || !mx || !my || !mz) return fail(MMC_ERR_INVALID, "null argument");
  TRY(set_dev(h));
  return get_m_impl(h, mx, my, mz);
}

int mmc_build_demag(mmc_handle* h, const char* cache_dir) {
  if (!h) return fail(MMC_ERR_INVALID, "null handle");
  if (!h->cfg.cal_demag_flag) return fail(MMC_ERR_STATE, "cal_demag_flag is off");
  if (h->demag_built) return MMC_OK;
  return build_demag_impl(h, cache_dir);
}

int mmc_get_tensor(mmc_handle* h, double* k6) {
  if (!h || !k6) return fail(MMC_ERR_INVALID, "null argument");
  TRY(set_dev(h));
  TRY(ensure_demag(h));
  if (!h->demag_built) return fail(MMC_ERR_STATE, "demag tensor not built (cal_demag_flag is off)");
  std::memcpy(k6, h->tensor.data(), h->tensor.size() * sizeof(double));
  return MMC_OK;
}

int mmc_self_tensor(mmc_handle* h, double k6[6]) {
  if (!h || !k6) return fail(MMC_ERR_INVALID, "null argument");
  TRY(set_dev(h));
  TRY(ensure_demag(h));
  if (!h->demag_built) return fail(MMC_ERR_STATE, "demag tensor not built (cal_demag_flag is off)");
  for (int q = 0; q < 6; ++q) k6[q] = h->k0[q];
  return MMC_OK;
}

int mmc_compute_demag(mmc_handle* h) {
  if (!h) return fail(MMC_ERR_INVALID, "null handle");
  if (!h->cfg.cal_demag_flag) return fail(MMC_ERR_STATE, "cal_demag_flag is off");
  TRY(set_dev(h));
  TRY(ensure_demag(h));
  CU(demag(h));
  return sync_check(h);
}

int mmc_demag_scratch_bytes(mmc_handle* h, size_t* bytes) {
  if (!h || !bytes) return fail(MMC_ERR_INVALID, "null argument");
  *bytes = 3 * (size_t)h->g.nspec * 2 * h->tsize;
  return MMC_OK;
}

int mmc_demag_apply(mmc_handle* h, const void* mdev, void* hdev, void* scratch, size_t scratch_bytes,
                    void* stream) {
  if (!h || !mdev || !hdev || !scratch) return fail(MMC_ERR_INVALID, "null argument");
  if (!h->cfg.cal_demag_flag) return fail(MMC_ERR_STATE, "cal_demag_flag is off");
  if (scratch_bytes < 3 * (size_t)h->g.nspec * 2 * h->tsize) return fail(MMC_ERR_INVALID, "scratch too small");
  TRY(set_dev(h));
  TRY(ensure_demag(h));
  cudaStream_t st = stream ? (cudaStream_t)stream : h->st;
  cudaError_t e = h->prec == 32 ? launch_demag<float>(h->g, h->px.p, h->py.p, h->pz.p, h->tun, (const float*)mdev,
                                                      (float*)hdev, scratch, h->khat, st)
                                : launch_demag<double>(h->g, h->px.p, h->py.p, h->pz.p, h->tun, (const double*)mdev,
                                                       (double*)hdev, scratch, h->khat, st);
  CU(e);
  return MMC_OK;
}

int mmc_demag_apply_static(mmc_handle* h, const void* mdev, void* hdev, void* stream) {
  if (!h || !mdev || !hdev) return fail(MMC_ERR_INVALID, "null argument");
  if (!h->cfg.cal_demag_flag) return fail(MMC_ERR_STATE, "cal_demag_flag is off");
  const size_t need = 3 * (size_t)h->g.nspec * 2 * h->tsize;
  if (need > (size_t)MMC_DEMAG_STATIC_SCRATCH_BYTES)
    return fail(MMC_ERR_INVALID, "this lattice's spectrum needs " + std::to_string(need) +
                                     " bytes, more than the static array's " +
                                     std::to_string((size_t)MMC_DEMAG_STATIC_SCRATCH_BYTES) +
                                     "; use mmc_demag_apply with caller scratch");
  if (!h->demag_built)
    return fail(MMC_ERR_STATE, "demag tensor not built: call mmc_build_demag first (building allocates)");
  TRY(set_dev(h));
  void* scratch = nullptr;
  CU(demag_static_scratch(h->device, &scratch));
  cudaStream_t st = stream ? (cudaStream_t)stream : h->st;
  cudaError_t e = h->prec == 32 ? launch_demag<float>(h->g, h->px.p, h->py.p, h->pz.p, h->tun, (const float*)mdev,
                                                      (float*)hdev, scratch, h->khat, st)
                                : launch_demag<double>(h->g, h->px.p, h->py.p, h->pz.p, h->tun, (const double*)mdev,
                                                       (double*)hdev, scratch, h->khat, st);
  CU(e);
  return MMC_OK;
}

int mmc_selftest_barrier_timeout(int device, long long spin_limit, int* status) {
  if (!status || spin_limit < 1 || spin_limit > (1ll << 24)) return fail(MMC_ERR_INVALID, "bad argument");
  CU(cudaSetDevice(device));
  void* bar = nullptr;
  int* ok = nullptr;
  CU(cudaMalloc(&bar, grid_barrier_bytes()));
  cudaError_t e = cudaMalloc(&ok, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(bar, 0, grid_barrier_bytes());
  if (e == cudaSuccess) e = cudaMemset(ok, 0xff, sizeof(int));
  if (e == cudaSuccess) e = launch_barrier_timeout_selftest(bar, (unsigned long long)spin_limit, ok);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  std::vector<unsigned char> hb(grid_barrier_bytes());
  int ok_host = -1;
  if (e == cudaSuccess) e = cudaMemcpy(hb.data(), bar, hb.size(), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&ok_host, ok, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(bar);
  if (ok) cudaFree(ok);
  CU(e);
  const bool timed_out = grid_barrier_error(reinterpret_cast<const GridBarrier*>(hb.data())) != 0 && ok_host == 0;
  *status = timed_out ? MMC_ERR_TIMEOUT : MMC_OK;
  return MMC_OK;
}

int mmc_selftest_mbar_timeout(int device, long long limit_ns, int* status) {
  if (!status || limit_ns < 1 || limit_ns > 1000000000ll) return fail(MMC_ERR_INVALID, "bad argument");
  CU(cudaSetDevice(device));
  int* flag = nullptr;
  CU(cudaMalloc(&flag, sizeof(int)));
  cudaError_t e = cudaMemset(flag, 0xff, sizeof(int));
  if (e == cudaSuccess) e = launch_mbar_timeout_selftest((unsigned long long)limit_ns, flag);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  int v = -1;
  if (e == cudaSuccess) e = cudaMemcpy(&v, flag, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(flag);
  CU(e);
  *status = v == 1 ? MMC_ERR_TIMEOUT : MMC_OK;
  return MMC_OK;
}

int mmc_selftest_philox(int device, long long n, const uint32_t* ctr, uint32_t k0, uint32_t k1, uint32_t* out,
                        uint32_t* out_curand) {
  if (n < 0 || (n > 0 && !ctr)) return fail(MMC_ERR_INVALID, "bad argument");
  if (n == 0) return MMC_OK;
  CU(cudaSetDevice(device));
  uint32_t* d = nullptr;
  CU(cudaMalloc(&d, 12 * (size_t)n * sizeof(uint32_t)));
  cudaError_t e = cudaMemcpy(d, ctr, 4 * (size_t)n * sizeof(uint32_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = launch_philox_selftest(n, d, k0, k1, d + 4 * n, d + 8 * n, nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess && out) e = cudaMemcpy(out, d + 4 * n, 4 * (size_t)n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && out_curand)
    e = cudaMemcpy(out_curand, d + 8 * n, 4 * (size_t)n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
  cudaFree(d);
  CU(e);
  return MMC_OK;
}

int mmc_get_field(mmc_handle* h, int term, double* hx, double* hy, double* hz) {
  if (!h || !hx || !hy || !hz) return fail(MMC_ERR_INVALID, "null argument");
  if (term < 0 || term > 5) return fail(MMC_ERR_INVALID, "bad term");
  TRY(set_dev(h));
  if ((term == MMC_TERM_DEMAG || term == MMC_TERM_TOTAL) && h->cfg.cal_demag_flag && !h->demag_built)
    return fail(MMC_ERR_STATE, "demag field not computed");
  HCoef k = make_h_coef(h);
  cudaError_t e = h->prec == 32 ? launch_field<float>(h->g, k, term, (const float*)h->m, (const float*)h->h,
                                                      h->field64, h->st)
                                : launch_field<double>(h->g, k, term, (const double*)h->m, (const double*)h->h,
                                                       h->field64, h->st);
  CU(e);
  const long long n = h->g.n;
  CU(cudaMemcpyAsync(hx, h->field64, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CU(cudaMemcpyAsync(hy, h->field64 + n, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CU(cudaMemcpyAsync(hz, h->field64 + 2 * n, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  return sync_check(h);
}

int mmc_grad(mmc_handle* h, double* dE_dm, double dE_dparams[7]) {
  if (!h || !dE_dparams) return fail(MMC_ERR_INVALID, "null argument");
  TRY(set_dev(h));
  return grad_impl(h, dE_dm, dE_dparams);
}

int mmc_relax(mmc_handle* h, double torque_tol, long long max_iter, long long* iters, double* max_torque) {
  if (!h) return fail(MMC_ERR_INVALID, "null handle");
  if (!(torque_tol > 0) || max_iter < 0) return fail(MMC_ERR_INVALID, "torque_tol must be > 0, max_iter >= 0");
  TRY(set_dev(h));
  h->stop.store(0);
  return relax_impl(h, torque_tol, max_iter, iters, max_torque);
}

int mmc_energy(mmc_handle* h, mmc_observables* out) {
  if (!h || !out) return fail(MMC_ERR_INVALID, "null argument");
  TRY(set_dev(h));
  return energy_impl(h, out);
}

int mmc_run_sweeps(mmc_handle* h, double temperature, long long stage, long long sweep0, long long nsweeps) {
  if (!h) return fail(MMC_ERR_INVALID, "null handle");
  if (!(temperature > 0)) return fail(MMC_ERR_INVALID, "temperature must be > 0");
  if (nsweeps < 0 || stage < 0 || sweep0 < 0) return fail(MMC_ERR_INVALID, "negative counter");
  TRY(set_dev(h));
  h->stop.store(0);
  return run_sweeps_impl(h, temperature, stage, sweep0, nsweeps);
}

int mmc_run_anneal(mmc_handle* h, const char* output_dir, int verbose) {
  if (!h || !output_dir) return fail(MMC_ERR_INVALID, "null argument");
  TRY(set_dev(h));
  h->stop.store(0);
  TRY(prepare_output_dir(output_dir));
  return h->prec == 32 ? anneal_loop<float>(h, output_dir, verbose) : anneal_loop<double>(h, output_dir, verbose);
}

int mmc_engine_info(mmc_handle* h, int out[3]) {
  if (!h || !out) return fail(MMC_ERR_INVALID, "null argument");
  out[0] = h->engine;
  out[1] = h->fused_band;
  out[2] = h->fused_blocks;
  return MMC_OK;
}

int mmc_profile_fused(mmc_handle* h, double temperature, long long stage, long long sweep0, long long nsweeps,
                      unsigned long long* stamps) {
  if (!h || !stamps) return fail(MMC_ERR_INVALID, "null argument");
  if (h->engine != MMC_ENGINE_FUSED) return fail(MMC_ERR_STATE, "the handle does not use the fused engine");
  if (nsweeps < 1 || nsweeps > 1024) return fail(MMC_ERR_INVALID, "nsweeps must be in [1, 1024]");
  TRY(set_dev(h));
  TRY(ensure_demag(h));
  TRY(upload_coef(h, temperature));
  unsigned long long* d = nullptr;
  CU(cudaMalloc(&d, FUSED_STAMP_WORDS * sizeof(unsigned long long)));
  cudaError_t e = cudaMemset(d, 0, FUSED_STAMP_WORDS * sizeof(unsigned long long));
  if (e == cudaSuccess)
    e = h->prec == 32 ? fused_chunk<float>(h, stage, sweep0, (int)nsweeps, d)
                      : fused_chunk<double>(h, stage, sweep0, (int)nsweeps, d);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  if (e == cudaSuccess)
    e = cudaMemcpy(stamps, d, FUSED_STAMP_WORDS * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaFree(d);
  CU(e);
  h->proposed += (unsigned long long)nsweeps * (unsigned long long)h->g.n;
  return MMC_OK;
}

int mmc_last_run_ms(mmc_handle* h, double* ms) {
  if (!h || !ms) return fail(MMC_ERR_INVALID, "null argument");
  *ms = h->last_run_ms;
  return MMC_OK;
}

int mmc_profile_sweeps(mmc_handle* h, double temperature, long long stage, long long sweep0, long long nsweeps,
                       double out_ms[3]) {
  if (!h || !out_ms) return fail(MMC_ERR_INVALID, "null argument");
  if (!(temperature > 0)) return fail(MMC_ERR_INVALID, "temperature must be > 0");
  TRY(set_dev(h));
  return profile_sweeps_impl(h, temperature, stage, sweep0, nsweeps, out_ms);
}


int mmc_batch_create(const mmc_config* cfgs, int nrep, int device, mmc_batch** out) {
  if (!cfgs || !out) return fail(MMC_ERR_INVALID, "null argument");
  return batch_create_impl(cfgs, nrep, device, out);
}

void mmc_batch_destroy(mmc_batch* b) { batch_free(b); }

int mmc_batch_size(mmc_batch* b) { return b ? b->R : 0; }

int mmc_batch_set_temperatures(mmc_batch* b, const double* T) {
  if (!b || !T) return fail(MMC_ERR_INVALID, "null argument");
  for (int r = 0; r < b->R; ++r)
    if (!(T[r] > 0)) return fail(MMC_ERR_INVALID, "temperatures must be > 0");
  b->T.assign(T, T + b->R);
  if (b->interval > 0) {
    TRY(set_dev(b->base));
    CU(cudaMemcpy(b->d_replica_T, b->T.data(), b->R * sizeof(double), cudaMemcpyHostToDevice));
  }
  return MMC_OK;
}

int mmc_batch_get_temperatures(mmc_batch* b, double* T) {
  if (!b || !T) return fail(MMC_ERR_INVALID, "null argument");
  TRY(set_dev(b->base));
  TRY(batch_sync_temperatures(b));
  std::memcpy(T, b->T.data(), b->R * sizeof(double));
  return MMC_OK;
}

int mmc_batch_set_ladders(mmc_batch* b, int nladders, int per_ladder, const int* replicas, const double* temps,
                          int swap_interval, long long seed) {
  if (!b || !replicas || !temps) return fail(MMC_ERR_INVALID, "null argument");
  if (nladders < 1 || per_ladder < 2 || (long long)nladders * per_ladder > b->R || swap_interval < 1)
    return fail(MMC_ERR_INVALID, "bad ladder shape");
  std::vector<int> seen(b->R, 0);
  for (int i = 0; i < nladders * per_ladder; ++i) {
    if (replicas[i] < 0 || replicas[i] >= b->R || seen[replicas[i]]++)
      return fail(MMC_ERR_INVALID, "ladder replicas must be distinct indices of the batch");
    if (!(temps[i] > 0)) return fail(MMC_ERR_INVALID, "ladder temperatures must be > 0");
  }
  TRY(set_dev(b->base));
  const size_t nk = (size_t)nladders * per_ladder;
  auto re = [&](void** p, size_t bytes) -> int {
    if (*p) cudaFree(*p);
    *p = nullptr;
    CU(cudaMalloc(p, bytes));
    return MMC_OK;
  };
  TRY(re((void**)&b->d_replica_at, nk * sizeof(int)));
  TRY(re((void**)&b->d_temps, nk * sizeof(double)));
  TRY(re((void**)&b->d_replica_T, b->R * sizeof(double)));
  TRY(re((void**)&b->d_round, sizeof(unsigned int)));
  TRY(re((void**)&b->d_counts, 2 * sizeof(unsigned long long)));
  for (size_t i = 0; i < nk; ++i) b->T[replicas[i]] = temps[i];
  CU(cudaMemcpy(b->d_replica_at, replicas, nk * sizeof(int), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(b->d_temps, temps, nk * sizeof(double), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(b->d_replica_T, b->T.data(), b->R * sizeof(double), cudaMemcpyHostToDevice));
  CU(cudaMemset(b->d_round, 0, sizeof(unsigned int)));
  CU(cudaMemset(b->d_counts, 0, 2 * sizeof(unsigned long long)));
  b->pt.nladders = nladders;
  b->pt.K = per_ladder;
  b->pt.replica_at = b->d_replica_at;
  b->pt.temps = b->d_temps;
  b->pt.replica_T = b->d_replica_T;
  b->pt.round = b->d_round;
  b->pt.counts = b->d_counts;
  b->pt.key0 = (uint32_t)((uint64_t)seed & 0xffffffffu);
  b->pt.key1 = (uint32_t)((uint64_t)seed >> 32);
  b->interval = swap_interval;
  batch_drop_graphs(b);
  return MMC_OK;
}

int mmc_batch_ladder_state(mmc_batch* b, int* replicas, unsigned long long counts[2]) {
  if (!b || b->interval <= 0) return fail(MMC_ERR_STATE, "no ladders set");
  TRY(set_dev(b->base));
  if (replicas)
    CU(cudaMemcpy(replicas, b->d_replica_at, (size_t)b->pt.nladders * b->pt.K * sizeof(int), cudaMemcpyDeviceToHost));
  if (counts) CU(cudaMemcpy(counts, b->d_counts, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  return MMC_OK;
}

int mmc_batch_run_sweeps(mmc_batch* b, long long stage, long long sweep0, long long nsweeps) {
  if (!b) return fail(MMC_ERR_INVALID, "null batch");
  if (nsweeps < 0 || stage < 0 || sweep0 < 0) return fail(MMC_ERR_INVALID, "negative counter");
  TRY(set_dev(b->base));
  b->stop.store(0);
  if (nsweeps == 0) return MMC_OK;
  return batch_run(b, stage, sweep0, nsweeps);
}

int mmc_batch_profile_sweeps(mmc_batch* b, long long stage, long long sweep0, long long nsweeps, double out_ms[5]) {
  if (!b || !out_ms) return fail(MMC_ERR_INVALID, "null argument");
  if (!b->base->cfg.cal_demag_flag) return fail(MMC_ERR_STATE, "cal_demag_flag is off");
  mmc_handle* h = b->base;
  TRY(set_dev(h));
  TRY(ensure_demag(h));
  TRY(batch_sync_temperatures(b));
  TRY(h->prec == 32 ? batch_upload_coefs<float>(b) : batch_upload_coefs<double>(b));
  CU(batch_set_counters(b, stage, sweep0));
  cudaEvent_t ev[5];
  for (auto& e : ev) CU(cudaEventCreate(&e));
  double acc[4] = {0, 0, 0, 0};
  int status = MMC_OK;
  if (b->rows_band > 0) {
    // film sweeps: [0] row kernel, [1] column pass
    cudaError_t e = batch_demag(b);
    for (long long s = 0; s < nsweeps && e == cudaSuccess; ++s) {
      e = batch_sweep_rows(b, (int)(s & 1), ev, 0);
      if (e == cudaSuccess) e = launch_advance(b->ctr, 1, h->st, CTR_SLOTS);
      if (e == cudaSuccess) e = cudaEventSynchronize(ev[2]);
      float x = 0, y = 0;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&x, ev[0], ev[1]);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&y, ev[1], ev[2]);
      acc[0] += x;
      acc[1] += y;
    }
    if (e == cudaSuccess && (nsweeps & 1)) e = batch_rows_settle(b);
    if (e != cudaSuccess) status = fail(MMC_ERR_CUDA, cudaGetErrorString(e));
  }
  for (long long s = 0; b->rows_band == 0 && s < nsweeps && status == MMC_OK; ++s) {
    cudaError_t e = batch_sweep(b, ev, 0, (int)(s & 1));
    if (e == cudaSuccess) e = launch_advance(b->ctr, 1, h->st, CTR_SLOTS);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[4]);
    for (int k = 0; k < 4 && e == cudaSuccess; ++k) {
      float ms = 0;
      e = cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
      acc[k] += ms;
    }
    if (e != cudaSuccess) status = fail(MMC_ERR_CUDA, cudaGetErrorString(e));
  }
  if (status == MMC_OK && batch_strip(b) && (nsweeps & 1)) {
    cudaError_t e = batch_strip_settle(b);
    if (e != cudaSuccess) status = fail(MMC_ERR_CUDA, cudaGetErrorString(e));
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (status != MMC_OK) return status;
  CU(cudaStreamSynchronize(h->st));
  for (int k = 0; k < 4; ++k) out_ms[k] = acc[k];
  out_ms[4] = acc[0] + acc[1] + acc[2] + acc[3];
  b->proposed += (unsigned long long)nsweeps * (unsigned long long)h->g.n;
  return MMC_OK;
}

int mmc_batch_set_launch_shape(mmc_batch* b, const int shape[10]) {
  if (!b || !shape) return fail(MMC_ERR_INVALID, "null argument");
  mmc_handle* h = b->base;
  const Geom& g = h->g;
  const size_t cs = 2 * h->tsize;
  DemagTuning t{shape[0], shape[1], shape[2], shape[3], shape[4], shape[6], shape[7], shape[8]};
  const int streams = shape[9];
  if (streams < 1 || streams > 4) return fail(MMC_ERR_INVALID, "streams must be in [1, 4]");
  const int band = shape[5];
  auto pow2 = [](int v) { return v > 0 && (v & (v - 1)) == 0; };
  if (!pow2(t.x_rows_per_cta) || t.x_rows_per_cta > 16 || x_pass_smem(h->px.p, t.x_rows_per_cta, cs) > smem_limit() ||
      !pow2(t.col_tx) || t.col_tx > 64 || col_pass_smem(h->py.p, t.col_tx, cs, t.col_lean != 0) > smem_limit() ||
      !pow2(t.col_tx_z) || t.col_tx_z > 64 || col_pass_smem(h->pz.p, t.col_tx_z, cs, t.col_lean != 0) > smem_limit() ||
      t.col_threads % t.col_tx != 0 ||
      t.col_threads % t.col_tx_z != 0 ||
      (t.x_threads != 128 && t.x_threads != 256) || t.col_threads < 32 || t.col_threads > 512 ||
      t.col_threads % 32 != 0 || t.mc_form < MC_FORM_SCALAR || t.mc_form > MC_FORM_PIPE ||
      (t.mc_form == MC_FORM_TILE && !mc_tile_eligible(g)) || (t.mc_form == MC_FORM_QUAD && !mc_quad_eligible(g)) ||
      (t.mc_form == MC_FORM_BAND && !mc_band_eligible(g)) ||
      (t.mc_form == MC_FORM_STRIP && (!mc_strip_eligible(g) || shape[5] != 0 ||
                                      mc_strip_smem_bytes(g, h->tsize) > smem_limit())) ||
      (t.mc_form == MC_FORM_PIPE && (!mc_pipe_eligible(g) || mc_pipe_smem_bytes(g, h->tsize) > smem_limit())) ||
      (t.fft_inline != 0 && t.fft_inline != 1) || t.col_lean < 0 || t.col_lean > 3)
    return fail(MMC_ERR_INVALID, "launch shape outside the supported range");
  if (band != 0 && std::find(b->row_bands.begin(), b->row_bands.end(), band) == b->row_bands.end())
    return fail(MMC_ERR_UNSUPPORTED, "row-kernel band not available for this batch");
  TRY(set_dev(h));
  if (band > 0) TRY(batch_alloc_rows(b));
  if (streams > 1) TRY(batch_alloc_streams(b));
  if (t.mc_form == MC_FORM_STRIP) TRY(batch_alloc_m2(b));
  b->tun = t;
  b->rows_band = band;
  b->streams = streams;
  batch_drop_graphs(b);
  return MMC_OK;
}

int mmc_batch_autotune(mmc_batch* b, int sweeps, double* best_ms_per_sweep, int* candidates) {
  if (!b) return fail(MMC_ERR_INVALID, "null batch");
  if (sweeps < 1 || sweeps > 100000) return fail(MMC_ERR_INVALID, "sweeps must be in [1, 100000]");
  TRY(set_dev(b->base));
  return batch_autotune(b, sweeps, best_ms_per_sweep, candidates);
}

int mmc_batch_launch_shape(mmc_batch* b, int out[10]) {
  if (!b || !out) return fail(MMC_ERR_INVALID, "null argument");
  out[9] = b->streams;
  out[5] = b->rows_band;
  out[6] = b->tun.mc_form;
  out[7] = b->tun.fft_inline;
  out[8] = b->tun.col_lean;
  out[0] = b->tun.x_rows_per_cta;
  out[1] = b->tun.x_threads;
  out[2] = b->tun.col_tx;
  out[3] = b->tun.col_tx_z;
  out[4] = b->tun.col_threads;
  return MMC_OK;
}

int mmc_batch_set_stream(mmc_batch* b, void* stream) {
  if (!b) return fail(MMC_ERR_INVALID, "null batch");
  return set_stream_impl(b->base, stream);
}

int mmc_batch_last_run_ms(mmc_batch* b, double* ms) {
  if (!b || !ms) return fail(MMC_ERR_INVALID, "null argument");
  *ms = b->last_ms;
  return MMC_OK;
}

// =================================================================== farms
// Several batches (one per lattice size, say) advanced together: their pieces
// are enqueued in turn on their own streams, so the GPU runs them
// concurrently.  The farm does not own its batches.
struct mmc_farm {
  std::vector<mmc_batch*> batches;
  double last_ms = 0;
  std::atomic<int> stop{0};
};

int mmc_farm_create(mmc_batch* const* batches, int nbatches, mmc_farm** out) {
  if (!batches || !out || nbatches < 1) return fail(MMC_ERR_INVALID, "need at least one batch");
  *out = nullptr;
  for (int i = 0; i < nbatches; ++i) {
    if (!batches[i]) return fail(MMC_ERR_INVALID, "null batch");
    if (batches[i]->base->device != batches[0]->base->device)
      return fail(MMC_ERR_INVALID, "the batches of a farm must share one device");
    for (int j = 0; j < i; ++j)
      if (batches[j] == batches[i]) return fail(MMC_ERR_INVALID, "a batch appears twice");
  }
  mmc_farm* f = new mmc_farm();
  f->batches.assign(batches, batches + nbatches);
  *out = f;
  return MMC_OK;
}

void mmc_farm_destroy(mmc_farm* f) { delete f; }

int mmc_farm_run_sweeps(mmc_farm* f, long long stage, long long sweep0, long long nsweeps) {
  if (!f) return fail(MMC_ERR_INVALID, "null farm");
  if (nsweeps < 0 || stage < 0 || sweep0 < 0) return fail(MMC_ERR_INVALID, "negative counter");
  TRY(set_dev(f->batches[0]->base));
  f->stop.store(0);
  const auto t0 = std::chrono::steady_clock::now();
  const size_t nb = f->batches.size();
  std::vector<BatchRun> runs(nb);
  for (size_t i = 0; i < nb; ++i) {
    f->batches[i]->stop.store(0);
    TRY(batch_run_begin(f->batches[i], runs[i], stage, sweep0, nsweeps));
  }
  std::vector<char> fin(nb, 0);
  for (long long round = 1;; ++round) {
    bool all = true;
    for (size_t i = 0; i < nb; ++i) {
      if (fin[i]) continue;
      bool done = false;
      TRY(batch_run_piece(f->batches[i], runs[i], &done));
      fin[i] = done;
      all = all && done;
    }
    if (f->stop.load()) return fail(MMC_ERR_INTERRUPTED, "stop requested");
    if (all) break;
    if (round % 32 == 0)
      for (size_t i = 0; i < nb; ++i) CU(cudaStreamSynchronize(f->batches[i]->base->st));
  }
  for (size_t i = 0; i < nb; ++i) TRY(batch_run_end(f->batches[i], runs[i]));
  f->last_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return MMC_OK;
}

int mmc_farm_last_run_ms(mmc_farm* f, double* ms) {
  if (!f || !ms) return fail(MMC_ERR_INVALID, "null argument");
  *ms = f->last_ms;
  return MMC_OK;
}

void mmc_farm_request_stop(mmc_farm* f) {
  if (f) f->stop.store(1);
}

void mmc_batch_request_stop(mmc_batch* b) {
  if (b) b->stop.store(1);
}

int mmc_batch_energy(mmc_batch* b, mmc_observables* out) {
  if (!b || !out) return fail(MMC_ERR_INVALID, "null argument");
  mmc_handle* h = b->base;
  TRY(set_dev(h));
  TRY(ensure_demag(h));
  CU(batch_energy_kernels(b));
  std::vector<unsigned long long> acc(b->R);
  CU(cudaMemcpyAsync(b->red_host, b->red, (size_t)b->R * NQ * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CU(cudaMemcpyAsync(acc.data(), b->acc, b->R * sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->st));
  CU(cudaStreamSynchronize(h->st));
  const double n = (double)h->g.n;
  for (int r = 0; r < b->R; ++r) {
    const double* q = b->red_host + (size_t)r * NQ;
    mmc_observables& o = out[r];
    o.e_exchange = q[0];
    o.e_dmi = q[1];
    o.e_anisotropy = q[2];
    o.e_zeeman = q[3];
    o.e_demag = q[4];
    o.e_total = q[0] + q[1] + q[2] + q[3] + q[4];
    o.m[0] = q[5] / n;
    o.m[1] = q[6] / n;
    o.m[2] = q[7] / n;
    o.q = q[8] / (4.0 * 3.14159265358979323846) / (double)h->g.nz;
    o.accepted = acc[r] - b->acc_base[r];
    o.proposed = b->proposed;
    b->acc_base[r] = acc[r];
  }
  b->proposed = 0;
  return MMC_OK;
}

int mmc_batch_set_m(mmc_batch* b, int r, const double* mx, const double* my, const double* mz) {
  if (!b || !mx || !my || !mz) return fail(MMC_ERR_INVALID, "null argument");
  size_t off;
  TRY(batch_replica_ptr(b, r, &off));
  mmc_handle* h = b->base;
  TRY(set_dev(h));
  const long long n = h->g.n;
  CU(cudaMemcpy(h->stage64, mx, n * sizeof(double), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(h->stage64 + n, my, n * sizeof(double), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(h->stage64 + 2 * n, mz, n * sizeof(double), cudaMemcpyHostToDevice));
  CU(h->prec == 32 ? launch_from_f64<float>(3 * n, h->stage64, (float*)b->m + off, h->st)
                   : launch_from_f64<double>(3 * n, h->stage64, (double*)b->m + off, h->st));
  CU(cudaStreamSynchronize(h->st));
  return MMC_OK;
}

int mmc_batch_get_m(mmc_batch* b, int r, double* mx, double* my, double* mz) {
  if (!b || !mx || !my || !mz) return fail(MMC_ERR_INVALID, "null argument");
  size_t off;
  TRY(batch_replica_ptr(b, r, &off));
  mmc_handle* h = b->base;
  TRY(set_dev(h));
  const long long n = h->g.n;
  CU(h->prec == 32 ? launch_to_f64<float>(3 * n, (const float*)b->m + off, h->stage64, h->st)
                   : launch_to_f64<double>(3 * n, (const double*)b->m + off, h->stage64, h->st));
  CU(cudaStreamSynchronize(h->st));
  CU(cudaMemcpy(mx, h->stage64, n * sizeof(double), cudaMemcpyDeviceToHost));
  CU(cudaMemcpy(my, h->stage64 + n, n * sizeof(double), cudaMemcpyDeviceToHost));
  CU(cudaMemcpy(mz, h->stage64 + 2 * n, n * sizeof(double), cudaMemcpyDeviceToHost));
  return MMC_OK;
}

}  // extern "C"

namespace {

// The stage loop of mmc_run_anneal for every replica of a batch at once: the
// schedule of replica 0 (all replicas must share it), one output folder per
// replica holding what a single run writes there.
template <typename R>
int batch_anneal_loop(mmc_batch* b, const std::string& dir, int verbose) {
  const mmc_config& c = b->cfgs[0];
  for (const mmc_config& q : b->cfgs)
    if (q.Temperature_start != c.Temperature_start || q.Temperature_end != c.Temperature_end ||
        q.Temperature_step != c.Temperature_step || q.Temperature_use_exp != c.Temperature_use_exp ||
        q.circle_per_stage != c.circle_per_stage || q.energy_output_period != c.energy_output_period ||
        q.ms_output_period != c.ms_output_period)
      return fail(MMC_ERR_INVALID, "batch anneals need one temperature schedule and output periods for all replicas");
  const int Rn = b->R;
  const mmc_handle* h = b->base;
  const long long n = h->g.n;
  std::vector<std::string> dirs(Rn), efiles(Rn);
  for (int r = 0; r < Rn; ++r) {
    char sub[32];
    std::snprintf(sub, sizeof sub, "replica_%03d", r);
    dirs[r] = join(dir, sub);
    TRY(prepare_output_dir(dirs[r]));
    efiles[r] = join(dirs[r], "energy.txt");
    FILE* fp = std::fopen(efiles[r].c_str(), "w");
    if (!fp) return fail(MMC_ERR_IO, "cannot create " + efiles[r]);
    std::fclose(fp);
  }
  std::vector<double> mm(3 * n), temps(Rn);
  std::vector<mmc_observables> obs(Rn);
  R T = (R)c.Temperature_start;
  const R Tend = (R)c.Temperature_end, Tstep = (R)c.Temperature_step;
  long long out_count = 0, stage = 0;
  while (T > Tend) {
    if (verbose) std::printf("\n\nTemperature: %.2f K (%d replicas)\n", (double)T, Rn);
    for (int r = 0; r < Rn; ++r) temps[r] = (double)T;
    TRY(mmc_batch_set_temperatures(b, temps.data()));
    long long s = 0;
    while (s < c.circle_per_stage) {
      if (b->stop.load()) return fail(MMC_ERR_INTERRUPTED, "stop requested");
      if (s % c.ms_output_period == 0) {
        for (int r = 0; r < Rn; ++r) {
          TRY(mmc_batch_get_m(b, r, mm.data(), mm.data() + n, mm.data() + 2 * n));
          char name[256];
          std::snprintf(name, sizeof name, "%06lld_%.2fK_%lld.ovf", out_count, (double)T, s);
          TRY(ovf_write(join(dirs[r], name), h->g.nx, h->g.ny, h->g.nz, b->cfgs[r].dx, b->cfgs[r].dy,
                        b->cfgs[r].dz, mm.data(), mm.data() + n, mm.data() + 2 * n, b->cfgs[r].ovf_format, "m"));
        }
        ++out_count;
      }
      if (s % c.energy_output_period == 0) {
        TRY(mmc_batch_energy(b, obs.data()));
        for (int r = 0; r < Rn; ++r) {
          FILE* fp = std::fopen(efiles[r].c_str(), "a");
          if (!fp) return fail(MMC_ERR_IO, "cannot append to " + efiles[r]);
          std::fprintf(fp, "%f %lld %g\n", (double)T, s, obs[r].e_total);
          std::fclose(fp);
        }
      }
      long long next = c.circle_per_stage;
      const long long per[2] = {c.ms_output_period, c.energy_output_period};
      for (long long p : per) next = std::min(next, (s / p + 1) * p);
      TRY(batch_run(b, stage, s, next - s));
      s = next;
    }
    T = c.Temperature_use_exp ? (R)(T * Tstep) : (R)(T - Tstep);
    ++stage;
  }
  if (verbose) std::printf("~~~~~~~~~~~~~~END~~~~~~~~~~~~~~~~~~~~~~~~~ \n");
  return MMC_OK;
}

}  // namespace

extern "C" {

int mmc_batch_run_anneal(mmc_batch* b, const char* output_dir, int verbose) {
  if (!b || !output_dir) return fail(MMC_ERR_INVALID, "null argument");
  TRY(set_dev(b->base));
  b->stop.store(0);
  TRY(prepare_output_dir(output_dir));
  return b->base->prec == 32 ? batch_anneal_loop<float>(b, output_dir, verbose)
                             : batch_anneal_loop<double>(b, output_dir, verbose);
}

int mmc_batch_build_demag(mmc_batch* b, const char* cache_dir) {
  if (!b) return fail(MMC_ERR_INVALID, "null batch");
  if (!b->base->cfg.cal_demag_flag) return fail(MMC_ERR_STATE, "cal_demag_flag is off");
  if (b->base->demag_built) return MMC_OK;
  return build_demag_impl(b->base, cache_dir);
}

void mmc_request_stop(mmc_handle* h) {
  if (h) h->stop.store(1);
}

int mmc_ovf_read(const char* path, int nx, int ny, int nz, double dx, double dy, double dz, double* mx, double* my,
                 double* mz) {
  if (!path || !mx || !my || !mz) return fail(MMC_ERR_INVALID, "null argument");
  return ovf_read(path, nx, ny, nz, dx, dy, dz, mx, my, mz);
}

int mmc_ovf_write(const char* path, int nx, int ny, int nz, double dx, double dy, double dz, const double* mx,
                  const double* my, const double* mz, int format, const char* title) {
  if (!path || !mx || !my || !mz) return fail(MMC_ERR_INVALID, "null argument");
  return ovf_write(path, nx, ny, nz, dx, dy, dz, mx, my, mz, format, title ? title : "m");
}

}  // extern "C"
