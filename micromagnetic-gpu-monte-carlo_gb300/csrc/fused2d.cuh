// fused2d.cuh -- persistent sweep kernel for films (nz = 1, two colours).
//
// One cooperative launch runs a chunk of sweeps.  CTA b owns a band of `band`
// consecutive rows and a fixed set of kx column pairs.  Per sweep there are two
// phases separated by grid barriers:
//
//   row phase    : 16-byte cp.async copies of the m rows y0-2 .. y1+1 and of
//                  the spectrum rows y0-1 .. y1 (band + one halo row per side),
//                  overlapped with the Philox proposals of the sweep;
//                  inverse x-FFT of those spectrum rows -> demag field h;
//                  colour-0 Metropolis updates of band + halo rows (the halo
//                  rows repeat, bit for bit, what their owners compute, so no
//                  barrier is needed before colour 1);
//                  colour-1 updates of the band rows;
//                  store m, forward x-FFT of the band rows -> spectrum rows.
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

namespace mmc {

// count is zeroed by the host before every launch; barrier k of the launch
// completes when count reaches k * gridDim.x.
struct GridBarrier {
  unsigned int count;
  unsigned int pad;
  int err;  // 0 ok, 1 a barrier wait ran out of its budget
  int pad2;
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded grid barrier.  Thread 0 publishes the CTA's arrival with a release
// reduction (no round trip) and polls the counter with acquire loads.
__device__ __forceinline__ bool grid_sync(GridBarrier* bar, unsigned int& target, int* flag_smem) {
  __syncthreads();
  if (threadIdx.x == 0) {
    target += gridDim.x;
    __threadfence();
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(&bar->count), "r"(1u) : "memory");
    unsigned long long spins = 0;
    int ok = 1;
    while (true) {
      unsigned int v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(&bar->count) : "memory");
      if ((int)(v - target) >= 0) break;
      if (++spins > (1ull << 24)) {  // seconds, far beyond any legitimate wait
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

// Shared-memory carve-up (bytes, 16-aligned).
struct Fused2DLayout {
  size_t twx, twy, kres, colraw, mrows, specraw, hrows, prop, fft, total;
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
  L.twx = align16((size_t)px.tw_total * cs);
  L.twy = align16((size_t)py.tw_total * cs);
  L.kres = align16((size_t)(L.resident ? L.resident : 1) * 6 * py.n * 2 * cs);
  L.colraw = align16((size_t)3 * g.ny * 2 * cs);
  L.mrows = align16((size_t)(band + 4) * 3 * g.nx * sizeof(T));
  L.specraw = align16((size_t)(band + 2) * 3 * g.hxp * cs);
  L.hrows = align16((size_t)(band + 2) * 3 * g.nx * sizeof(T));
  L.prop = align16((size_t)(2 * band + 2) * ((g.nx + 1) / 2) * 4 * sizeof(T));
  const size_t xl = (size_t)2 * (band + 2) * px.n;
  const size_t yl = (size_t)6 * (py.n + 1);
  L.fft = align16((xl > yl ? xl : yl) * cs);
  L.total = L.twx + L.twy + L.kres + L.colraw + L.mrows + L.specraw + L.hrows + L.prop + 2 * L.fft;
  return L;
}

__device__ __forceinline__ int fused_row(int r, int ny, int per) {
  if (r < 0 || r >= ny) {
    if (!per) return -1;
    r = ((r % ny) + ny) % ny;
  }
  return r;
}

template <typename T>
__global__ void __launch_bounds__(FUSED_THREADS, 1) k_fused2d(Fused2D<T> P) {
  using V = C<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_flag;
  __shared__ int s_rows[64];  // slot -> row (or -1); slot k holds row y0 - 2 + k
  __shared__ unsigned int s_acc;
  const Geom& g = P.g;
  const int nx = g.nx, ny = g.ny, L = P.px.n, hx = g.hx, hxp = g.hxp, Ly = P.py.n;
  const long long n = g.n, nspec = g.nspec;
  const int G = gridDim.x;
  const Fused2DLayout lay = fused2d_layout<T>(g, P.px, P.py, P.band, G);
  unsigned char* ptr = smem_raw;
  V* twx = reinterpret_cast<V*>(ptr);
  ptr += lay.twx;
  V* twy = reinterpret_cast<V*>(ptr);
  ptr += lay.twy;
  V* kres = reinterpret_cast<V*>(ptr);  // [item][comp][ky][2]
  ptr += lay.kres;
  V* colraw = reinterpret_cast<V*>(ptr);  // [comp][y][2]
  ptr += lay.colraw;
  T* msm = reinterpret_cast<T*>(ptr);  // [slot][comp][x]
  ptr += lay.mrows;
  V* specraw = reinterpret_cast<V*>(ptr);  // [work][comp][kx]
  ptr += lay.specraw;
  T* hsm = reinterpret_cast<T*>(ptr);  // [work][comp][x]
  ptr += lay.hrows;
  Proposal<T>* prop = reinterpret_cast<Proposal<T>*>(ptr);
  ptr += lay.prop;
  V* fa = reinterpret_cast<V*>(ptr);
  ptr += lay.fft;
  V* fb = reinterpret_cast<V*>(ptr);

  const McCoef<T> c = *P.coef;
  unsigned int target = 0;
  const bool timed = P.tbuf && threadIdx.x == 0 && (blockIdx.x == 0 || blockIdx.x == G - 1);
  const int tcol = blockIdx.x == 0 ? 0 : 1;
  auto stamp = [&](int sw, int point) {
    if (timed && sw >= 0 && sw < FUSED_TSWEEPS) P.tbuf[((size_t)sw * FUSED_TPOINTS + point) * 2 + tcol] = global_ns();
  };

  const int y0 = blockIdx.x * P.band;
  const int nb = max(0, min(P.band, ny - y0));  // own rows: slots 2 .. nb+1
  const int nslots = nb + 4;
  const int nwork = nb + 2;                     // work rows: slots 1 .. nb+2
  const int half = (nx + 1) >> 1;
  const size_t mstride = 3 * (size_t)nx;
  const int elems = 16 / (int)sizeof(T);        // m values per 16-byte copy
  const int per_m = nx / elems;                 // 16-byte copies per component row of m
  const int ve = 16 / (int)sizeof(V);           // spectrum values per 16-byte copy
  const int per_s = hxp / ve;                   // 16-byte copies per component row of S
  if (threadIdx.x < nslots) s_rows[threadIdx.x] = fused_row(y0 - 2 + (int)threadIdx.x, ny, g.per[1]);
  if (threadIdx.x == 0) s_acc = 0;
  load_twiddles<T>(P.px, twx);
  load_twiddles<T>(P.py, twy);
  // resident tensor spectrum of the owned kx pairs
  for (int it = 0; it < lay.resident; ++it) {
    const int j = blockIdx.x + it * G;
    if (j >= lay.npairs) break;
    for (int idx = threadIdx.x; idx < 6 * Ly; idx += blockDim.x) {
      const int cc = idx / Ly, ky = idx - cc * Ly;
      for (int q = 0; q < 2 / ve; ++q)
        cp_async16(kres + (((size_t)it * 6 + cc) * Ly + ky) * 2 + q * ve,
                   P.K + cc * nspec + (long long)ky * hxp + 2 * j + q * ve);
    }
  }
  cp_async_wait_all();
  __syncthreads();

  // forward x-FFT of the band rows held in msm -> spectrum rows in global memory
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
    V* res = fft_run<T, false>(fa, fb, 2 * nb, L, P.px, twx);
    for (int idx = threadIdx.x; idx < nb * hx; idx += blockDim.x) {
      const int rr = idx / hx, k = idx - rr * hx;
      const V* la = res + (size_t)(2 * rr) * L;
      const V* lb = la + L;
      const int kn = k == 0 ? 0 : L - k;
      const V A = la[k], B = la[kn];
      const V A2 = lb[k], B2 = lb[kn];
      const long long off = (long long)(y0 + rr) * hxp + k;
      P.S[off] = cmk<V>((T)0.5 * (A.x + B.x), (T)0.5 * (A.y - B.y));
      P.S[nspec + off] = cmk<V>((T)0.5 * (A.y + B.y), (T)-0.5 * (A.x - B.x));
      P.S[2 * nspec + off] = cmk<V>((T)0.5 * (A2.x + B2.x), (T)0.5 * (A2.y - B2.y));
    }
  };

  // y-FFT, tensor product, inverse y-FFT for the owned kx pairs
  auto column_phase = [&](int sw) {
    for (int it = 0; it < lay.items; ++it) {
      const int j = blockIdx.x + it * G;
      if (j >= lay.npairs) break;
      const int kx0 = 2 * j;
      for (int idx = threadIdx.x; idx < 3 * ny; idx += blockDim.x) {
        const int cc = idx / ny, y = idx - cc * ny;
        for (int q = 0; q < 2 / ve; ++q)
          cp_async16(colraw + ((size_t)cc * ny + y) * 2 + q * ve, P.S + cc * nspec + (long long)y * hxp + kx0 + q * ve);
      }
      const V* kp = kres + (size_t)it * 6 * Ly * 2;
      if (!lay.resident) {  // stream K^ into kres (room for one item)
        for (int idx = threadIdx.x; idx < 6 * Ly; idx += blockDim.x) {
          const int cc = idx / Ly, ky = idx - cc * Ly;
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
        const int line = idx / Ly, pos = idx - line * Ly;
        const int cc = line >> 1, t = line & 1;
        fa[(size_t)line * (Ly + 1) + pos] = pos < ny ? colraw[((size_t)cc * ny + pos) * 2 + t] : cmk<V>(0, 0);
      }
      __syncthreads();
      V* cur = fft_run<T, false>(fa, fb, 6, Ly + 1, P.py, twy);
      V* oth = cur == fa ? fb : fa;
      for (int idx = threadIdx.x; idx < 2 * Ly; idx += blockDim.x) {
        const int t = idx / Ly, pos = idx - t * Ly;
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
        const int cc = idx / ny, y = idx - cc * ny;
        V* dst = P.S + cc * nspec + (long long)y * hxp + kx0;
        dst[0] = r[(size_t)(2 * cc) * (Ly + 1) + y];
        dst[1] = r[(size_t)(2 * cc + 1) * (Ly + 1) + y];
      }
      __syncthreads();
    }
  };

  // prologue: spectrum of the initial m
  for (int idx = threadIdx.x; idx < nb * 3 * per_m; idx += blockDim.x) {
    const int rr = idx / (3 * per_m), rem = idx - rr * 3 * per_m;
    const int cc = rem / per_m, q = rem - cc * per_m;
    cp_async16(msm + (size_t)(rr + 2) * mstride + (size_t)cc * nx + q * elems,
               P.m + cc * n + (long long)(y0 + rr) * nx + q * elems);
  }
  cp_async_wait_all();
  __syncthreads();
  x_forward_band();
  if (!grid_sync(P.bar, target, &s_flag)) return;
  column_phase(-1);
  if (!grid_sync(P.bar, target, &s_flag)) return;

  unsigned int my_acc = 0;
  for (int sw = 0; sw < P.nsweeps; ++sw) {
    const uint32_t sweep = P.sweep0 + (uint32_t)sw;
    const bool last = sw == P.nsweeps - 1;
    stamp(sw, 0);
    // m rows of every slot, spectrum rows of the work slots: 16-byte async copies
    for (int idx = threadIdx.x; idx < nslots * 3 * per_m; idx += blockDim.x) {
      const int slot = idx / (3 * per_m), rem = idx - slot * 3 * per_m;
      const int r = s_rows[slot];
      if (r < 0) continue;
      const int cc = rem / per_m, q = rem - cc * per_m;
      cp_async16(msm + (size_t)slot * mstride + (size_t)cc * nx + q * elems,
                 P.m + cc * n + (long long)r * nx + q * elems);
    }
    for (int idx = threadIdx.x; idx < nwork * 3 * per_s; idx += blockDim.x) {
      const int w = idx / (3 * per_s), rem = idx - w * 3 * per_s;
      const int r = s_rows[w + 1];
      if (r < 0) continue;
      const int cc = rem / per_s, q = rem - cc * per_s;
      cp_async16(specraw + ((size_t)w * 3 + cc) * hxp + q * ve, P.S + cc * nspec + (long long)r * hxp + q * ve);
    }
    // Philox proposals while the copies are in flight: colour 0 of the work
    // rows, then colour 1 of the band rows
    for (int idx = threadIdx.x; idx < (nwork + nb) * half; idx += blockDim.x) {
      const int k = idx / half, j = idx - k * half;
      const int color = k < nwork ? 0 : 1;
      const int slot = color == 0 ? 1 + k : 2 + (k - nwork);
      const int y = s_rows[slot];
      if (y < 0) continue;
      const int x = 2 * j + ((color + y) & 1);
      if (x >= nx) continue;
      prop[idx] = mc_propose<T>(c, (uint32_t)(x + nx * y), P.stage, sweep);
    }
    cp_async_wait_all();
    __syncthreads();
    stamp(sw, 1);
    // inverse x-FFT of the work rows -> h
    for (int idx = threadIdx.x; idx < nwork * L; idx += blockDim.x) {
      const int w = idx / L, k = idx - w * L;
      V A = cmk<V>(0, 0), B = cmk<V>(0, 0);
      if (s_rows[w + 1] >= 0) {
        const bool lo = k < hx;
        const int kk = lo ? k : L - k;
        const V* sr = specraw + (size_t)w * 3 * hxp;
        V v0 = sr[kk], v1 = sr[hxp + kk], v2 = sr[2 * hxp + kk];
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
      V* res = fft_run<T, true>(fa, fb, 2 * nwork, L, P.px, twx);
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
    stamp(sw, 2);
    // colour 0 on work rows, colour 1 on band rows
    for (int color = 0; color < 2; ++color) {
      const int kbase = color == 0 ? 0 : nwork;
      const int kcnt = color == 0 ? nwork : nb;
      for (int idx = threadIdx.x; idx < kcnt * half; idx += blockDim.x) {
        const int k = kbase + idx / half, j = idx - (idx / half) * half;
        const int slot = color == 0 ? 1 + k : 2 + (k - nwork);
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
        const Proposal<T> p = prop[k * half + j];
        if (mc_accept<T>(c, nbv, row[x], row[nx + x], row[2 * nx + x], hr[x], hr[nx + x], hr[2 * nx + x], p)) {
          row[x] = p.x;
          row[nx + x] = p.y;
          row[2 * nx + x] = p.z;
          if (slot >= 2 && slot < 2 + nb) my_acc += 1;
        }
      }
      __syncthreads();
    }
    stamp(sw, 3);
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
    stamp(sw, 4);
    if (!grid_sync(P.bar, target, &s_flag)) return;
    stamp(sw, 5);
    column_phase(sw);
    stamp(sw, 7);
    if (!grid_sync(P.bar, target, &s_flag)) return;
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

template <typename T>
cudaError_t fused2d_blocks_per_sm(const Geom& g, const FftPlan& px, const FftPlan& py, int band, int* out) {
  const size_t smem = fused2d_smem_bytes<T>(g, px, py, band);
  cudaError_t e =
      cudaFuncSetAttribute((const void*)k_fused2d<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
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
  P.h = a.h;
  P.S = reinterpret_cast<C<T>*>(a.spec);
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

#define MMC_INSTANTIATE_FUSED(T)                                                                                \
  template size_t fused2d_smem_bytes<T>(const Geom&, const FftPlan&, const FftPlan&, int);                     \
  template cudaError_t fused2d_blocks_per_sm<T>(const Geom&, const FftPlan&, const FftPlan&, int, int*);       \
  template cudaError_t launch_fused2d<T>(const Geom&, const FftPlan&, const FftPlan&, const FusedArgs<T>&, int, \
                                         cudaStream_t);

}  // namespace mmc
