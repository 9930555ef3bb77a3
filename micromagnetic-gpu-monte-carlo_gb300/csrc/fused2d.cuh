// fused2d.cuh -- persistent sweep kernel for films (nz = 1, two colours).
//
// One cooperative launch runs a chunk of sweeps.  CTA b owns a band of `band`
// consecutive rows and a fixed set of kx column pairs.  Per sweep there are two
// phases separated by grid barriers:
//
//   row phase    : the shared row phase of rows.cuh -- inverse x-FFT of the
//                  band's spectrum rows (plus one halo row per side), colour 0
//                  on band + halo rows, colour 1 on the band rows, store m,
//                  forward x-FFT of the band rows;
//   column phase : for each owned kx pair: y-FFT, the 3x3 tensor product
//                  (K^ . M^ / N, calHexchangeKernel of the reference,
//                  src/demag_cu.cu:68-116) with K^ kept resident in shared
//                  memory, inverse y-FFT.
//
// This is the reference's per-sweep sequence (demag refresh, then the
// Metropolis kernel, src/main.cu:868-884, 1101-1120) with the transforms and
// both colours fused; fields and decisions are bit-identical to the
// multi-kernel path (same FFT code, same mc_propose / mc_accept).  Data written
// by other CTAs is read only through L2 (cp.async.cg).  Barrier waits are
// bounded: on timeout the kernel records an error and returns.
#pragma once
#include "kernels.cuh"
#include "rows.cuh"

namespace mmc {

// count is zeroed by the host before every launch; barrier k of the launch
// completes when count reaches k * gridDim.x.
struct GridBarrier {
  unsigned int count;
  unsigned int pad;
  int err;  // 0 ok, 1 a barrier wait ran out of its budget
  int pad2;
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded grid barrier.  Thread 0 publishes the CTA's arrival with a release
// reduction (no round trip) and polls the counter with acquire loads.
// spin_limit: polls before the wait gives up (the default is seconds, far
// beyond any legitimate wait); expect: arrivals this barrier waits for.
// The barrier in two halves: grid_arrive publishes this CTA's arrival (after
// all its threads' writes), grid_wait polls until every CTA has arrived.  Work
// that needs nothing from other CTAs can run between the two.
__device__ __forceinline__ void grid_arrive(GridBarrier* bar, unsigned int& target, unsigned int expect = 0) {
  __syncthreads();
  if (threadIdx.x == 0) {
    target += expect ? expect : gridDim.x;
    __threadfence();
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(&bar->count), "r"(1u) : "memory");
  }
}

__device__ __forceinline__ bool grid_wait(GridBarrier* bar, unsigned int target, int* flag_smem,
                                          unsigned long long spin_limit = 1ull << 24) {
  if (threadIdx.x == 0) {
    unsigned long long spins = 0;
    int ok = 1;
    while (true) {
      unsigned int v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(&bar->count) : "memory");
      if ((int)(v - target) >= 0) break;
      if (++spins > spin_limit) {
        atomicExch(&bar->err, 1);
        ok = 0;
        break;
      }
      if (spins > 256) __nanosleep(32);
    }
    *flag_smem = ok;
  }
  __syncthreads();
  return *flag_smem != 0;
}

__device__ __forceinline__ bool grid_sync(GridBarrier* bar, unsigned int& target, int* flag_smem,
                                          unsigned long long spin_limit = 1ull << 24, unsigned int expect = 0) {
  grid_arrive(bar, target, expect);
  return grid_wait(bar, target, flag_smem, spin_limit);
}

template <typename T>
struct Fused2D {
  Geom g;
  FftPlan px, py;
  const McCoef<T>* coef;
  T* m;   // m; holds the result after an even number of sweeps
  T* m2;  // second copy of m; holds the result after an odd number
  T* h;
  C<T>* S;
  C<T>* S2;
  const C<T>* K;
  unsigned long long* acc;
  GridBarrier* bar;
  unsigned long long* tbuf;  // optional phase timestamps (CTA 0 and the last CTA)
  uint32_t stage, sweep0;
  int nsweeps;
  int band;
  T inv_n;
};

constexpr int FUSED_THREADS = 256;
constexpr int FUSED_MAX_RES = 2;   // kx pairs whose K^ stays resident in shared memory
constexpr int FUSED_TPOINTS = 9;   // timestamps per sweep
constexpr int FUSED_TSWEEPS = 16;  // sweeps recorded

// Shared-memory carve-up (bytes, 16-aligned): the row phase's buffers (its
// transform buffers sized for the column phase too), then the y twiddles, the
// resident tensor spectrum and the column staging area.
struct Fused2DLayout {
  size_t rowph, twy, kres, colraw, total;
  int npairs, items, resident;
};

__host__ __device__ inline size_t align16(size_t b) { return (b + 15) & ~(size_t)15; }

template <typename T>
__host__ __device__ inline Fused2DLayout fused2d_layout(const Geom& g, const FftPlan& px, const FftPlan& py, int band,
                                                        int nblocks) {
  Fused2DLayout L;
  const size_t cs = sizeof(C<T>);
  L.npairs = g.hxp / 2;
  L.items = (L.npairs + nblocks - 1) / nblocks;
  L.resident = L.items <= FUSED_MAX_RES ? L.items : 0;
  L.rowph = row_phase_bytes<T>(g, px, band, true, (size_t)6 * (py.n + 1));
  L.twy = align16((size_t)py.tw_total * cs);
  L.kres = align16((size_t)(L.resident ? L.resident : 1) * 6 * py.n * 2 * cs);
  L.colraw = align16((size_t)3 * g.ny * 2 * cs);
  L.total = L.rowph + L.twy + L.kres + L.colraw;
  return L;
}

template <typename T>
__global__ void __launch_bounds__(FUSED_THREADS, 1) k_fused2d(const __grid_constant__ Fused2D<T> P) {
  using V = C<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_flag;
  __shared__ int s_rows[64];  // slot -> row (or -1); slot k holds row y0 - 2 + k
  __shared__ unsigned int s_acc;
  const Geom& g = P.g;
  const int ny = g.ny, hxp = g.hxp, Ly = P.py.n;
  const long long nspec = g.nspec;
  const int G = gridDim.x;
  const Fused2DLayout lay = fused2d_layout<T>(g, P.px, P.py, P.band, G);
  RowPhase<T> R;
  R.g = g;
  R.px = &P.px;
  unsigned char* ptr = smem_raw;
  row_phase_carve<T>(R, ptr, P.band, true, (size_t)6 * (Ly + 1));
  V* twy = reinterpret_cast<V*>(ptr);
  ptr += lay.twy;
  V* kres = reinterpret_cast<V*>(ptr);  // [item][comp][ky][2]
  ptr += lay.kres;
  V* colraw = reinterpret_cast<V*>(ptr);  // [comp][y][2]
  V* fa = R.fa;
  V* fb = R.fb;
  R.rows = s_rows;
  R.h = P.h;
  R.y0 = blockIdx.x * P.band;
  R.nb = max(0, min(P.band, ny - R.y0));

  const McCoef<T> c = *P.coef;
  unsigned int target = 0;
  const bool timed = P.tbuf && threadIdx.x == 0 && (blockIdx.x == 0 || blockIdx.x == G - 1);
  const int tcol = blockIdx.x == 0 ? 0 : 1;
  auto stamp = [&](int sw, int point) {
    if (timed && sw >= 0 && sw < FUSED_TSWEEPS) P.tbuf[((size_t)sw * FUSED_TPOINTS + point) * 2 + tcol] = global_ns();
  };
  const int nb = R.nb;
  const int ve = 16 / (int)sizeof(V);  // spectrum values per 16-byte copy
  if (threadIdx.x < nb + 4) s_rows[threadIdx.x] = band_row(R.y0 - 2 + (int)threadIdx.x, ny, g.per[1]);
  if (threadIdx.x == 0) s_acc = 0;
  load_twiddles<T>(P.px, R.twx);
  load_twiddles<T>(P.py, twy);
  // resident tensor spectrum of the owned kx pairs
  for (int it = 0; it < lay.resident; ++it) {
    const int j = blockIdx.x + it * G;
    if (j >= lay.npairs) break;
    for (int idx = threadIdx.x; idx < 6 * Ly; idx += blockDim.x) {
      const int cc = P.py.dn.div(idx), ky = idx - cc * Ly;
      for (int q = 0; q < 2 / ve; ++q)
        cp_async16(kres + (((size_t)it * 6 + cc) * Ly + ky) * 2 + q * ve,
                   P.K + cc * nspec + (long long)ky * hxp + 2 * j + q * ve);
    }
  }
  cp_async_wait_all();
  __syncthreads();

  // y-FFT, tensor product, inverse y-FFT for the owned kx pairs of spectrum S
  auto column_phase = [&](int sw, C<T>* S) {
    for (int it = 0; it < lay.items; ++it) {
      const int j = blockIdx.x + it * G;
      if (j >= lay.npairs) break;
      const int kx0 = 2 * j;
      for (int idx = threadIdx.x; idx < 3 * ny; idx += blockDim.x) {
        const int cc = g.dny.div(idx), y = idx - cc * ny;
        for (int q = 0; q < 2 / ve; ++q)
          cp_async16(colraw + ((size_t)cc * ny + y) * 2 + q * ve, S + cc * nspec + (long long)y * hxp + kx0 + q * ve);
      }
      const V* kp = kres + (size_t)it * 6 * Ly * 2;
      if (!lay.resident) {  // stream K^ into kres (room for one item)
        for (int idx = threadIdx.x; idx < 6 * Ly; idx += blockDim.x) {
          const int cc = P.py.dn.div(idx), ky = idx - cc * Ly;
          for (int q = 0; q < 2 / ve; ++q)
            cp_async16(kres + ((size_t)cc * Ly + ky) * 2 + q * ve, P.K + cc * nspec + (long long)ky * hxp + kx0 + q * ve);
        }
        kp = kres;
      }
      cp_async_wait_all();
      __syncthreads();
      if (it == 0) stamp(sw, 6);
      // lines (comp, t) of length Ly with stride Ly + 1
      for (int idx = threadIdx.x; idx < 6 * Ly; idx += blockDim.x) {
        const int line = P.py.dn.div(idx), pos = idx - line * Ly;
        const int cc = line >> 1, t = line & 1;
        fa[(size_t)line * (Ly + 1) + pos] = pos < ny ? colraw[((size_t)cc * ny + pos) * 2 + t] : cmk<V>(0, 0);
      }
      __syncthreads();
      V* cur = fft_run<T, false>(fa, fb, 6, Ly + 1, P.py, twy);
      V* oth = cur == fa ? fb : fa;
      for (int idx = threadIdx.x; idx < 2 * Ly; idx += blockDim.x) {
        const int t = P.py.dn.div(idx), pos = idx - t * Ly;
        const V* kk = kp + (size_t)pos * 2 + t;
        const size_t ks = (size_t)Ly * 2;
        const V kxx = kk[0], kxy = kk[ks], kxz = kk[2 * ks], kyy = kk[3 * ks], kyz = kk[4 * ks], kzz = kk[5 * ks];
        V* qx = cur + (size_t)(0 + t) * (Ly + 1) + pos;
        V* qy = cur + (size_t)(2 + t) * (Ly + 1) + pos;
        V* qz = cur + (size_t)(4 + t) * (Ly + 1) + pos;
        const V mx = *qx, my = *qy, mz = *qz;
        T hxr = (mx.x * kxx.x - mx.y * kxx.y) + (my.x * kxy.x - my.y * kxy.y) + (mz.x * kxz.x - mz.y * kxz.y);
        T hxi = (mx.x * kxx.y + mx.y * kxx.x) + (my.x * kxy.y + my.y * kxy.x) + (mz.x * kxz.y + mz.y * kxz.x);
        T hyr = (mx.x * kxy.x - mx.y * kxy.y) + (my.x * kyy.x - my.y * kyy.y) + (mz.x * kyz.x - mz.y * kyz.y);
        T hyi = (mx.x * kxy.y + mx.y * kxy.x) + (my.x * kyy.y + my.y * kyy.x) + (mz.x * kyz.y + mz.y * kyz.x);
        T hzr = (mx.x * kxz.x - mx.y * kxz.y) + (my.x * kyz.x - my.y * kyz.y) + (mz.x * kzz.x - mz.y * kzz.y);
        T hzi = (mx.x * kxz.y + mx.y * kxz.x) + (my.x * kyz.y + my.y * kyz.x) + (mz.x * kzz.y + mz.y * kzz.x);
        *qx = cmk<V>(hxr * P.inv_n, hxi * P.inv_n);
        *qy = cmk<V>(hyr * P.inv_n, hyi * P.inv_n);
        *qz = cmk<V>(hzr * P.inv_n, hzi * P.inv_n);
      }
      __syncthreads();
      V* r = fft_run<T, true>(cur, oth, 6, Ly + 1, P.py, twy);
      for (int idx = threadIdx.x; idx < 3 * ny; idx += blockDim.x) {
        const int cc = g.dny.div(idx), y = idx - cc * ny;
        V* dst = S + cc * nspec + (long long)y * hxp + kx0;
        dst[0] = r[(size_t)(2 * cc) * (Ly + 1) + y];
        dst[1] = r[(size_t)(2 * cc + 1) * (Ly + 1) + y];
      }
      __syncthreads();
    }
  };

  // prologue: spectrum of the initial m
  {
    const int nx = g.nx;
    const int elems = 16 / (int)sizeof(T), per_m = nx / elems;
    for (int idx = threadIdx.x; idx < nb * 3 * per_m; idx += blockDim.x) {
      const int rr = idx / (3 * per_m), rem = idx - rr * 3 * per_m;
      const int cc = rem / per_m, q = rem - cc * per_m;
      cp_async16(R.msm + (size_t)(rr + 2) * 3 * nx + (size_t)cc * nx + q * elems,
                 P.m + cc * g.n + (long long)(R.y0 + rr) * nx + q * elems);
    }
    cp_async_wait_all();
    __syncthreads();
  }
  R.So = P.S;
  row_forward<T>(R);
  if (!grid_sync(P.bar, target, &s_flag)) return;
  column_phase(-1, P.S);
  if (!grid_sync(P.bar, target, &s_flag)) return;

  unsigned int my_acc = 0;
  for (int sw = 0; sw < P.nsweeps; ++sw) {
    const uint32_t sweep = P.sweep0 + (uint32_t)sw;
    const bool last = sw == P.nsweeps - 1;
    // even sweeps (m, S) -> (m2, S2), odd sweeps back
    R.m = (sw & 1) ? P.m2 : P.m;
    R.mo = (sw & 1) ? P.m : P.m2;
    R.S = (sw & 1) ? P.S2 : P.S;
    R.So = (sw & 1) ? P.S : P.S2;
    stamp(sw, 0);
    row_load<T>(R, c, P.stage, sweep, sw == 0);  // later sweeps' proposals were made during barrier 2
    stamp(sw, 1);
    row_field<T>(R);
    stamp(sw, 2);
    my_acc += row_sweep<T>(R, c);
    stamp(sw, 3);
    row_store<T>(R, last);
    if (last) break;
    row_forward<T>(R);
    stamp(sw, 4);
    if (!grid_sync(P.bar, target, &s_flag)) return;
    stamp(sw, 5);
    column_phase(sw, R.So);
    stamp(sw, 7);
    // the next sweep's proposals depend on nothing other CTAs write: make them
    // while the barrier's arrivals come in
    grid_arrive(P.bar, target);
    row_proposals<T>(R, c, P.stage, sweep + 1);
    if (!grid_wait(P.bar, target, &s_flag)) return;
    stamp(sw, 8);
  }
  unsigned int v = my_acc;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(&s_acc, v);
  __syncthreads();
  if (threadIdx.x == 0 && s_acc) atomicAdd(P.acc, (unsigned long long)s_acc);
}

template <typename T>
size_t fused2d_smem_bytes(const Geom& g, const FftPlan& px, const FftPlan& py, int band) {
  const int nblocks = (g.ny + band - 1) / band;
  return fused2d_layout<T>(g, px, py, band, nblocks).total;
}

// The kernels' dynamic shared-memory limit is raised to the device's opt-in
// maximum once, not to one lattice's need: the attribute is per kernel and
// process-wide, so a later, smaller lattice must not lower it under an
// earlier one.
// The opt-in maximum covers static and dynamic shared memory together.
inline cudaError_t raise_smem_limit(const void* fn) {
  int dev = 0, optin = 48 * 1024;
  cudaFuncAttributes fa{};
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, fn);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
  return e;
}

template <typename T>
cudaError_t fused2d_blocks_per_sm(const Geom& g, const FftPlan& px, const FftPlan& py, int band, int* out) {
  const size_t smem = fused2d_smem_bytes<T>(g, px, py, band);
  cudaError_t e = raise_smem_limit((const void*)k_fused2d<T>);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, (const void*)k_fused2d<T>, FUSED_THREADS, smem);
}

template <typename T>
cudaError_t launch_fused2d(const Geom& g, const FftPlan& px, const FftPlan& py, const FusedArgs<T>& a, int nblocks,
                           cudaStream_t st) {
  Fused2D<T> P;
  P.g = g;
  P.px = px;
  P.py = py;
  P.coef = a.coef;
  P.m = a.m;
  P.m2 = a.m2;
  P.h = a.h;
  P.S = reinterpret_cast<C<T>*>(a.spec);
  P.S2 = reinterpret_cast<C<T>*>(a.spec2);
  if (!a.m2 || !a.spec2 || a.m2 == a.m || a.spec2 == a.spec) return cudaErrorInvalidValue;
  P.K = reinterpret_cast<const C<T>*>(a.khat);
  P.acc = a.acc;
  P.bar = a.bar;
  P.tbuf = a.tbuf;
  P.stage = a.stage;
  P.sweep0 = a.sweep0;
  P.nsweeps = a.nsweeps;
  P.band = a.band;
  P.inv_n = (T)(1.0 / (double)g.np);
  const size_t smem = fused2d_layout<T>(g, px, py, a.band, nblocks).total;
  cudaError_t e = cudaMemsetAsync(&a.bar->count, 0, sizeof(unsigned int), st);
  if (e != cudaSuccess) return e;
  void* args[] = {(void*)&P};
  return cudaLaunchCooperativeKernel((const void*)k_fused2d<T>, dim3(nblocks), dim3(FUSED_THREADS), args, smem, st);
}

// ------------------------------------------------------- batched film sweeps
template <typename T>
size_t rows_smem_bytes(const Geom& g, const FftPlan& px, int band) {
  return row_phase_bytes<T>(g, px, band, px.warp_a == 0);
}

template <typename T>
cudaError_t rows_prepare(const Geom& g, const FftPlan& px, int band, int* blocks_per_sm) {
  const size_t smem = rows_smem_bytes<T>(g, px, band);
  cudaError_t e = raise_smem_limit((const void*)k_rows<T>);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, (const void*)k_rows<T>, 256, smem);
}

template <typename T>
cudaError_t launch_rows(const Geom& g, const FftPlan& px, const McCoef<T>* coef, const T* m, T* mo, T* h,
                        const void* spec, void* spec_out, unsigned long long* acc, const SweepCounters* ctr, int band,
                        int nrep, bool with_h, bool do_forward, cudaStream_t st) {
  if (m == mo || spec == spec_out) return cudaErrorInvalidValue;  // halo rows must not be overwritten
  const size_t smem = rows_smem_bytes<T>(g, px, band);
  dim3 grid((g.ny + band - 1) / band, 1, nrep);
  k_rows<T><<<grid, 256, smem, st>>>(g, px, coef, m, mo, h, reinterpret_cast<const C<T>*>(spec),
                                     reinterpret_cast<C<T>*>(spec_out), acc, ctr, band, with_h ? 1 : 0,
                                     do_forward ? 1 : 0);
  return cudaGetLastError();
}

#define MMC_INSTANTIATE_FUSED(T)                                                                                \
  template size_t fused2d_smem_bytes<T>(const Geom&, const FftPlan&, const FftPlan&, int);                     \
  template cudaError_t fused2d_blocks_per_sm<T>(const Geom&, const FftPlan&, const FftPlan&, int, int*);       \
  template cudaError_t launch_fused2d<T>(const Geom&, const FftPlan&, const FftPlan&, const FusedArgs<T>&, int, \
                                         cudaStream_t);                                                        \
  template size_t rows_smem_bytes<T>(const Geom&, const FftPlan&, int);                                        \
  template cudaError_t rows_prepare<T>(const Geom&, const FftPlan&, int, int*);                                \
  template cudaError_t launch_rows<T>(const Geom&, const FftPlan&, const McCoef<T>*, const T*, T*, T*,        \
                                      const void*, void*, unsigned long long*, const SweepCounters*, int, int, bool, \
                                      bool, cudaStream_t);

}  // namespace mmc
