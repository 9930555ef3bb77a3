// fused2d.cuh -- persistent sweep kernel for films (nz = 1, two colours).
//
// One cooperative launch runs a chunk of sweeps.  CTA b owns a band of
// `band` consecutive rows; per sweep there are two phases separated by grid
// barriers:
//
//   row phase    : inverse x-FFT of the band's spectrum rows plus one halo row
//                  on each side -> demag field h of those rows;
//                  colour-0 Metropolis updates of band + halo rows (the halo
//                  rows repeat, bit for bit, what their owners compute, so no
//                  barrier is needed before colour 1);
//                  colour-1 updates of the band rows;
//                  store m, forward x-FFT of the band rows -> spectrum rows.
//   column phase : for each kx column: y-FFT, the 3x3 tensor product
//                  (K^ . M^ / N, calHexchangeKernel of the reference,
//                  src/demag_cu.cu:68-116), inverse y-FFT.
//
// This is the reference's per-sweep sequence (demag refresh, then the
// Metropolis kernel, src/main.cu:868-884, 1101-1120) with the transforms and
// both colours fused; decisions and fields are bit-identical to the
// multi-kernel path (same FFT code, same mc_decide).  Data written by other
// CTAs is read with L2-coherent loads (__ldcg).  Every barrier wait is
// bounded: on timeout the kernel records an error and returns.
#pragma once
#include "kernels.cuh"

namespace mmc {

struct GridBarrier {
  unsigned int count;
  unsigned int gen;
  int err;       // 0 ok, 1 barrier timeout
  int pad;
};

// Bounded sense-by-generation barrier over gridDim.x co-resident CTAs.
// Returns false (for every thread of the CTA) when any CTA has timed out.
__device__ __forceinline__ bool grid_sync(GridBarrier* bar, unsigned int& gen, int* flag_smem) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned int arrived = atomicAdd(&bar->count, 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(&bar->count, 0u);
      __threadfence();
      atomicAdd(&bar->gen, 1u);
    } else {
      unsigned long long spins = 0;
      while (true) {
        unsigned int g;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(g) : "l"(&bar->gen) : "memory");
        if (g != gen) break;
        if (++spins > (1ull << 24)) {  // ~1-2 s with the back-off below
          atomicExch(&bar->err, 1);
          break;
        }
        if (spins > 64) __nanosleep(64);
      }
    }
    __threadfence();
    gen += 1;
    *flag_smem = *((volatile int*)&bar->err);
  }
  __syncthreads();
  return *flag_smem == 0;
}

template <typename T>
struct Fused2D {
  Geom g;
  FftPlan px, py;
  const McCoef<T>* coef;
  T* m;
  T* h;
  C<T>* S;
  const C<T>* K;
  unsigned long long* acc;
  GridBarrier* bar;
  uint32_t stage, sweep0;
  int nsweeps;
  int band;
  int have_spectrum;  // 1: S already holds the spectrum of m (skip the prologue)
  T inv_n;
};

// Shared-memory carve-up for a given band (all sizes in bytes, 16-aligned).
struct Fused2DLayout {
  size_t twx, twy, mrows, hrows, fft, total;
};

__host__ __device__ inline size_t align16(size_t b) { return (b + 15) & ~(size_t)15; }

template <typename T>
__host__ __device__ inline Fused2DLayout fused2d_layout(const Geom& g, const FftPlan& px, const FftPlan& py, int band) {
  Fused2DLayout L;
  const size_t cs = sizeof(C<T>);
  L.twx = align16((size_t)px.tw_total * cs);
  L.twy = align16((size_t)py.tw_total * cs);
  L.mrows = align16((size_t)(band + 4) * 3 * g.nx * sizeof(T));
  L.hrows = align16((size_t)(band + 2) * 3 * g.nx * sizeof(T));
  size_t xl = (size_t)2 * (band + 2) * px.n;  // x-pass lines, complex elements
  size_t yl = (size_t)3 * (py.n + 1);
  L.fft = align16((xl > yl ? xl : yl) * cs);
  L.total = L.twx + L.twy + L.mrows + L.hrows + 2 * L.fft;
  return L;
}

template <typename T>
__device__ __forceinline__ int wrap_row(int r, int ny, int per, bool* ok) {
  if (r < 0 || r >= ny) {
    if (!per) {
      *ok = false;
      return 0;
    }
    r = ((r % ny) + ny) % ny;
  }
  *ok = true;
  return r;
}

template <typename T>
__global__ void __launch_bounds__(256) k_fused2d(Fused2D<T> P) {
  using V = C<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_flag;
  __shared__ int s_rows[64];  // slot -> row (or -1)
  __shared__ unsigned int s_acc;
  const Geom& g = P.g;
  const int nx = g.nx, ny = g.ny, L = P.px.n, hx = g.hx, Ly = P.py.n;
  const long long n = g.n, nspec = g.nspec;
  Fused2DLayout lay = fused2d_layout<T>(g, P.px, P.py, P.band);
  unsigned char* ptr = smem_raw;
  V* twx = reinterpret_cast<V*>(ptr);
  ptr += lay.twx;
  V* twy = reinterpret_cast<V*>(ptr);
  ptr += lay.twy;
  T* msm = reinterpret_cast<T*>(ptr);  // [slot][c][x]
  ptr += lay.mrows;
  T* hsm = reinterpret_cast<T*>(ptr);  // [work slot - 1][c][x]
  ptr += lay.hrows;
  V* fa = reinterpret_cast<V*>(ptr);
  ptr += lay.fft;
  V* fb = reinterpret_cast<V*>(ptr);

  const McCoef<T> c = *P.coef;
  load_twiddles<T>(P.px, twx);
  load_twiddles<T>(P.py, twy);
  unsigned int gen = 0;
  if (threadIdx.x == 0) gen = *((volatile unsigned int*)&P.bar->gen);

  const int y0 = blockIdx.x * P.band;
  const int nb = max(0, min(P.band, ny - y0));  // own rows
  const int nslots = nb + 4;                    // rows y0-2 .. y0+nb+1
  if (threadIdx.x < nslots) {
    bool ok;
    int r = wrap_row<T>(y0 - 2 + (int)threadIdx.x, ny, g.per[1], &ok);
    s_rows[threadIdx.x] = ok ? r : -1;
  }
  if (threadIdx.x == 0) s_acc = 0;
  __syncthreads();
  const size_t mstride = 3 * (size_t)nx;  // per slot
  const int ncols = hx;

  // ------------------------------------------------ helpers
  // forward x-FFT of the band rows held in msm slots 2..nb+1 -> S rows
  auto x_forward_band = [&]() {
    for (int idx = threadIdx.x; idx < nb * L; idx += blockDim.x) {
      const int rr = idx / L, x = idx - rr * L;
      const T* row = msm + (size_t)(rr + 2) * mstride;
      V a = cmk<V>(0, 0), b = cmk<V>(0, 0);
      if (x < nx) {
        a = cmk<V>(row[x], row[nx + x]);
        b = cmk<V>(row[2 * nx + x], (T)0);
      }
      fa[(size_t)(2 * rr) * L + x] = a;
      fa[(size_t)(2 * rr + 1) * L + x] = b;
    }
    __syncthreads();
    V* res = fft_lines<T, false>(fa, fb, 2 * nb, L, P.px, twx);
    for (int idx = threadIdx.x; idx < nb * 2 * hx; idx += blockDim.x) {
      const int k = idx % hx;
      const int rest = idx / hx;
      const int pr = rest % 2, rr = rest / 2;
      const V* line = res + (size_t)(2 * rr + pr) * L;
      const V A = line[k];
      const V B = line[k == 0 ? 0 : L - k];
      const long long off = (long long)(y0 + rr) * hx + k;
      if (pr == 0) {
        P.S[off] = cmk<V>((T)0.5 * (A.x + B.x), (T)0.5 * (A.y - B.y));
        P.S[nspec + off] = cmk<V>((T)0.5 * (A.y + B.y), (T)-0.5 * (A.x - B.x));
      } else {
        P.S[2 * nspec + off] = cmk<V>((T)0.5 * (A.x + B.x), (T)0.5 * (A.y - B.y));
      }
    }
  };

  // column phase: y-FFT, tensor product, inverse y-FFT for columns b, b+G, ...
  auto column_phase = [&]() {
    for (int col = blockIdx.x; col < ncols; col += gridDim.x) {
      for (int idx = threadIdx.x; idx < 3 * Ly; idx += blockDim.x) {
        const int pos = idx % Ly, cc = idx / Ly;
        V v = cmk<V>(0, 0);
        if (pos < ny) v = __ldcg(&P.S[cc * nspec + (long long)pos * hx + col]);
        fa[(size_t)cc * (Ly + 1) + pos] = v;
      }
      __syncthreads();
      V* cur = fft_lines<T, false>(fa, fb, 3, Ly + 1, P.py, twy);
      V* oth = cur == fa ? fb : fa;
      for (int pos = threadIdx.x; pos < Ly; pos += blockDim.x) {
        const long long ka = (long long)pos * hx + col;
        const V kxx = P.K[ka], kxy = P.K[nspec + ka], kxz = P.K[2 * nspec + ka];
        const V kyy = P.K[3 * nspec + ka], kyz = P.K[4 * nspec + ka], kzz = P.K[5 * nspec + ka];
        V* qx = cur + pos;
        V* qy = cur + (Ly + 1) + pos;
        V* qz = cur + 2 * (Ly + 1) + pos;
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
      V* r = fft_lines<T, true>(cur, oth, 3, Ly + 1, P.py, twy);
      for (int idx = threadIdx.x; idx < 3 * ny; idx += blockDim.x) {
        const int pos = idx % ny, cc = idx / ny;
        P.S[cc * nspec + (long long)pos * hx + col] = r[(size_t)cc * (Ly + 1) + pos];
      }
      __syncthreads();
    }
  };

  // ------------------------------------------------ prologue: spectrum of m
  if (!P.have_spectrum) {
    for (int idx = threadIdx.x; idx < nb * (int)mstride; idx += blockDim.x) {
      const int rr = idx / (int)mstride, rem = idx - rr * (int)mstride;
      const int cc = rem / nx, x = rem - cc * nx;
      msm[(size_t)(rr + 2) * mstride + rem] = __ldcg(&P.m[cc * n + (long long)(y0 + rr) * nx + x]);
    }
    __syncthreads();
    x_forward_band();
    if (!grid_sync(P.bar, gen, &s_flag)) return;
    column_phase();
    if (!grid_sync(P.bar, gen, &s_flag)) return;
  }

  unsigned int my_acc = 0;
  for (int sw = 0; sw < P.nsweeps; ++sw) {
    const uint32_t sweep = P.sweep0 + (uint32_t)sw;
    const bool last = sw == P.nsweeps - 1;
    // -------- row phase: load m rows of all slots, spectrum rows of work slots
    for (int idx = threadIdx.x; idx < nslots * (int)mstride; idx += blockDim.x) {
      const int slot = idx / (int)mstride, rem = idx - slot * (int)mstride;
      const int r = s_rows[slot];
      if (r < 0) continue;
      const int cc = rem / nx, x = rem - cc * nx;
      msm[idx] = __ldcg(&P.m[cc * n + (long long)r * nx + x]);
    }
    const int nwork = nb + 2;  // slots 1 .. nb+2
    for (int idx = threadIdx.x; idx < nwork * L; idx += blockDim.x) {
      const int w = idx / L, k = idx - w * L;
      const int r = s_rows[w + 1];
      V A = cmk<V>(0, 0), B = cmk<V>(0, 0);
      if (r >= 0) {
        const bool lo = k < hx;
        const long long kk = lo ? k : L - k;
        const long long base = (long long)r * hx + kk;
        V v0 = __ldcg(&P.S[base]), v1 = __ldcg(&P.S[nspec + base]), v2 = __ldcg(&P.S[2 * nspec + base]);
        if (!lo) {
          v0.y = -v0.y;
          v1.y = -v1.y;
          v2.y = -v2.y;
        }
        if (k == 0 || 2 * k == L) v0.y = v1.y = v2.y = 0;
        A = cmk<V>(v0.x - v1.y, v0.y + v1.x);
        B = v2;
      }
      fa[(size_t)(2 * w) * L + k] = A;
      fa[(size_t)(2 * w + 1) * L + k] = B;
    }
    __syncthreads();
    {
      V* res = fft_lines<T, true>(fa, fb, 2 * nwork, L, P.px, twx);
      for (int idx = threadIdx.x; idx < nwork * nx; idx += blockDim.x) {
        const int w = idx / nx, x = idx - w * nx;
        const V a = res[(size_t)(2 * w) * L + x];
        const V b = res[(size_t)(2 * w + 1) * L + x];
        T* hr = hsm + (size_t)w * mstride;
        hr[x] = a.x;
        hr[nx + x] = a.y;
        hr[2 * nx + x] = b.x;
      }
    }
    __syncthreads();
    // colour 0 on band + halo rows, colour 1 on band rows
    for (int color = 0; color < 2; ++color) {
      const int s_lo = color == 0 ? 1 : 2;
      const int s_cnt = color == 0 ? nwork : nb;
      const int half = (nx + 1) >> 1;
      for (int idx = threadIdx.x; idx < s_cnt * half; idx += blockDim.x) {
        const int slot = s_lo + idx / half;
        const int j = idx - (idx / half) * half;
        const int y = s_rows[slot];
        if (y < 0) continue;
        const int x = 2 * j + ((color + y) & 1);
        if (x >= nx) continue;
        T* row = msm + (size_t)slot * mstride;
        Nbrs<T> nbv;
#pragma unroll
        for (int s = 0; s < 2; ++s) {
          int xx = x + (s ? 1 : -1);
          bool ok = true;
          if (xx < 0 || xx >= nx) {
            if (g.per[0]) xx = xx < 0 ? xx + nx : xx - nx;
            else ok = false;
          }
          if (xx == x) ok = false;
          nbv.has[0][s] = ok;
          const int xs = ok ? xx : x;
          nbv.v[0][s][0] = row[xs];
          nbv.v[0][s][1] = row[nx + xs];
          nbv.v[0][s][2] = row[2 * nx + xs];
          const int ns = slot + (s ? 1 : -1);
          const bool oky = s_rows[ns] >= 0 && s_rows[ns] != y;
          nbv.has[1][s] = oky;
          const T* r2 = msm + (size_t)(oky ? ns : slot) * mstride;
          nbv.v[1][s][0] = r2[x];
          nbv.v[1][s][1] = r2[nx + x];
          nbv.v[1][s][2] = r2[2 * nx + x];
          nbv.has[2][s] = false;
          nbv.v[2][s][0] = nbv.v[2][s][1] = nbv.v[2][s][2] = (T)0;
        }
        const T* hr = hsm + (size_t)(slot - 1) * mstride;
        T qx, qy, qz;
        if (mc_decide<T>(c, nbv, row[x], row[nx + x], row[2 * nx + x], hr[x], hr[nx + x], hr[2 * nx + x],
                         (uint32_t)(x + nx * y), P.stage, sweep, qx, qy, qz)) {
          row[x] = qx;
          row[nx + x] = qy;
          row[2 * nx + x] = qz;
          if (slot >= 2 && slot < 2 + nb) my_acc += 1;
        }
      }
      __syncthreads();
    }
    // store the band's m (and h after the last sweep)
    for (int idx = threadIdx.x; idx < nb * (int)mstride; idx += blockDim.x) {
      const int rr = idx / (int)mstride, rem = idx - rr * (int)mstride;
      const int cc = rem / nx, x = rem - cc * nx;
      const long long gi = cc * n + (long long)(y0 + rr) * nx + x;
      P.m[gi] = msm[(size_t)(rr + 2) * mstride + rem];
      if (last) P.h[gi] = hsm[(size_t)(rr + 1) * mstride + rem];
    }
    if (last) break;
    x_forward_band();
    if (!grid_sync(P.bar, gen, &s_flag)) return;
    column_phase();
    if (!grid_sync(P.bar, gen, &s_flag)) return;
  }
  // accept count: warp-aggregate then one atomic per CTA
  unsigned int v = my_acc;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(&s_acc, v);
  __syncthreads();
  if (threadIdx.x == 0 && s_acc) atomicAdd(P.acc, (unsigned long long)s_acc);
}

template <typename T>
size_t fused2d_smem_bytes(const Geom& g, const FftPlan& px, const FftPlan& py, int band) {
  return fused2d_layout<T>(g, px, py, band).total;
}

template <typename T>
cudaError_t fused2d_blocks_per_sm(const Geom& g, const FftPlan& px, const FftPlan& py, int band, int* out) {
  const size_t smem = fused2d_smem_bytes<T>(g, px, py, band);
  cudaError_t e =
      cudaFuncSetAttribute((const void*)k_fused2d<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, (const void*)k_fused2d<T>, 256, smem);
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
  P.h = a.h;
  P.S = reinterpret_cast<C<T>*>(a.spec);
  P.K = reinterpret_cast<const C<T>*>(a.khat);
  P.acc = a.acc;
  P.bar = a.bar;
  P.stage = a.stage;
  P.sweep0 = a.sweep0;
  P.nsweeps = a.nsweeps;
  P.band = a.band;
  P.have_spectrum = 0;
  P.inv_n = (T)(1.0 / (double)g.np);
  const size_t smem = fused2d_smem_bytes<T>(g, px, py, a.band);
  void* args[] = {(void*)&P};
  return cudaLaunchCooperativeKernel((const void*)k_fused2d<T>, dim3(nblocks), dim3(256), args, smem, st);
}

#define MMC_INSTANTIATE_FUSED(T)                                                                                \
  template size_t fused2d_smem_bytes<T>(const Geom&, const FftPlan&, const FftPlan&, int);                     \
  template cudaError_t fused2d_blocks_per_sm<T>(const Geom&, const FftPlan&, const FftPlan&, int, int*);       \
  template cudaError_t launch_fused2d<T>(const Geom&, const FftPlan&, const FftPlan&, const FusedArgs<T>&, int, \
                                         cudaStream_t);

}  // namespace mmc
