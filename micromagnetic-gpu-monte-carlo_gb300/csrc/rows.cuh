// rows.cuh -- the row phase of a film sweep, shared by the persistent film
// engine (fused2d.cuh) and the batched row kernel (k_rows).
//
// For a band of rows y0 .. y0+nb-1 of one film (nz = 1, two colours), with the
// spectrum S already holding K^ . M^ / N of the current m:
//   copy   : m rows y0-2 .. y0+nb+1 and spectrum rows y0-1 .. y0+nb into
//            shared memory with 16-byte cp.async copies, Philox proposals of
//            the sweep computed while they land;
//   field  : inverse x-FFT of the spectrum rows -> demag field h of the band
//            and one halo row per side;
//   sweep  : colour 0 on band + halo rows (the halo rows repeat, bit for bit,
//            what their owners compute), then colour 1 on the band rows;
//   store  : the band's m, optionally h;
//   forward: x-FFT of the updated band rows -> spectrum rows.
// Reads come from (m, S) and writes go to (mo, So), distinct buffers: other
// bands read this band's rows as their halo during the same sweep, so the
// sweeps alternate between two copies of m and of the spectrum.
// Slot k of the shared row cache holds row y0 - 2 + k (wrapped on a periodic
// axis, -1 outside an open one).
#pragma once
#include "kernels.cuh"

namespace mmc {

__device__ __forceinline__ int band_row(int r, int ny, int per) {
  if (r < 0 || r >= ny) {
    if (!per) return -1;
    r = ((r % ny) + ny) % ny;
  }
  return r;
}

template <typename T>
struct RowPhase {
  Geom g;
  const FftPlan* px;
  C<T>* twx;
  T* msm;            // [slot][comp][x], slots 0 .. nb+3
  C<T>* specraw;     // [work][comp][kx], work rows = slots 1 .. nb+2
  T* hsm;            // [work][comp][x]
  Proposal<T>* prop; // colour 0 of the work rows, then colour 1 of the band rows
  C<T>* fa;
  C<T>* fb;
  const int* rows;   // slot -> row
  const T* m;    // m at the start of the sweep
  T* mo;         // m after the sweep (band rows)
  T* h;
  const C<T>* S; // spectrum rows of the start-of-sweep field
  C<T>* So;      // spectrum rows of the updated band
  int y0, nb;
};

// Shared-memory bytes of the row phase for a band (16-aligned pieces).
template <typename T>
__host__ __device__ inline size_t row_phase_bytes(const Geom& g, const FftPlan& px, int band, bool two_fft,
                                                  size_t min_fft = 0) {
  const size_t cs = sizeof(C<T>);
  auto a16 = [](size_t b) { return (b + 15) & ~(size_t)15; };
  size_t b = a16((size_t)px.tw_total * cs);
  b += a16((size_t)(band + 4) * 3 * g.nx * sizeof(T));
  b += a16((size_t)(band + 2) * 3 * g.hxp * cs);
  b += a16((size_t)(band + 2) * 3 * g.nx * sizeof(T));
  b += a16((size_t)(2 * band + 2) * ((g.nx + 1) / 2) * 4 * sizeof(T));
  size_t fl = (size_t)2 * (band + 2) * px.n;
  if (fl < min_fft) fl = min_fft;
  b += (two_fft ? 2 : 1) * a16(fl * cs);
  return b;
}

// Carves the row-phase buffers out of `ptr` (advanced past them).
template <typename T>
__device__ __forceinline__ void row_phase_carve(RowPhase<T>& R, unsigned char*& ptr, int band, bool two_fft,
                                                size_t min_fft = 0) {
  const size_t cs = sizeof(C<T>);
  auto a16 = [](size_t b) { return (b + 15) & ~(size_t)15; };
  R.twx = reinterpret_cast<C<T>*>(ptr);
  ptr += a16((size_t)R.px->tw_total * cs);
  R.msm = reinterpret_cast<T*>(ptr);
  ptr += a16((size_t)(band + 4) * 3 * R.g.nx * sizeof(T));
  R.specraw = reinterpret_cast<C<T>*>(ptr);
  ptr += a16((size_t)(band + 2) * 3 * R.g.hxp * cs);
  R.hsm = reinterpret_cast<T*>(ptr);
  ptr += a16((size_t)(band + 2) * 3 * R.g.nx * sizeof(T));
  R.prop = reinterpret_cast<Proposal<T>*>(ptr);
  ptr += a16((size_t)(2 * band + 2) * ((R.g.nx + 1) / 2) * 4 * sizeof(T));
  size_t fe = (size_t)2 * (band + 2) * R.px->n;
  if (fe < min_fft) fe = min_fft;
  const size_t fl = a16(fe * cs);
  R.fa = reinterpret_cast<C<T>*>(ptr);
  ptr += fl;
  R.fb = two_fft ? reinterpret_cast<C<T>*>(ptr) : R.fa;
  if (two_fft) ptr += fl;
}

// Philox proposals of the sweep for colour 0 on the work rows and colour 1 on
// the band rows (they depend only on cell, stage and sweep).
template <typename T>
__device__ __forceinline__ void row_proposals(const RowPhase<T>& R, const McCoef<T>& c, uint32_t stage,
                                              uint32_t sweep) {
  const int nx = R.g.nx, nwork = R.nb + 2, half = (nx + 1) >> 1;
  for (int idx = threadIdx.x; idx < (nwork + R.nb) * half; idx += blockDim.x) {
    const int k = R.g.dhxc.div(idx), j = idx - k * half;
    const int color = k < nwork ? 0 : 1;
    const int slot = color == 0 ? 1 + k : 2 + (k - nwork);
    const int y = R.rows[slot];
    if (y < 0) continue;
    const int x = 2 * j + ((color + y) & 1);
    if (x >= nx) continue;
    R.prop[idx] = mc_propose<T>(c, (uint32_t)(x + nx * y), stage, sweep);
  }
}

// copy (+ proposals, while the copies land); ends with the data in shared
// memory, after __syncthreads
template <typename T>
__device__ __forceinline__ void row_load(const RowPhase<T>& R, const McCoef<T>& c, uint32_t stage, uint32_t sweep,
                                         bool with_proposals = true) {
  using V = C<T>;
  const int nx = R.g.nx, hxp = R.g.hxp;
  const long long n = R.g.n, nspec = R.g.nspec;
  const int nslots = R.nb + 4, nwork = R.nb + 2;
  const size_t mstride = 3 * (size_t)nx;
  const int elems = 16 / (int)sizeof(T), per_m = nx / elems;
  const int ve = 16 / (int)sizeof(V), per_s = hxp / ve;
  const FastDiv d3m((uint32_t)(3 * per_m)), dm((uint32_t)per_m), d3s((uint32_t)(3 * per_s)), ds((uint32_t)per_s);
  for (int idx = threadIdx.x; idx < nslots * 3 * per_m; idx += blockDim.x) {
    const int slot = d3m.div(idx), rem = idx - slot * 3 * per_m;
    const int r = R.rows[slot];
    if (r < 0) continue;
    const int cc = dm.div(rem), q = rem - cc * per_m;
    cp_async16(R.msm + (size_t)slot * mstride + (size_t)cc * nx + q * elems, R.m + cc * n + (long long)r * nx + q * elems);
  }
  for (int idx = threadIdx.x; idx < nwork * 3 * per_s; idx += blockDim.x) {
    const int w = d3s.div(idx), rem = idx - w * 3 * per_s;
    const int r = R.rows[w + 1];
    if (r < 0) continue;
    const int cc = ds.div(rem), q = rem - cc * per_s;
    cp_async16(R.specraw + ((size_t)w * 3 + cc) * hxp + q * ve, R.S + cc * nspec + (long long)r * hxp + q * ve);
  }
  if (with_proposals) row_proposals<T>(R, c, stage, sweep);
  cp_async_wait_all();
  __syncthreads();
}

// inverse x-FFT of the work rows -> hsm
template <typename T>
__device__ __forceinline__ void row_field(const RowPhase<T>& R) {
  using V = C<T>;
  const int nx = R.g.nx, hx = R.g.hx, hxp = R.g.hxp, L = R.px->n;
  const int nwork = R.nb + 2;
  const size_t mstride = 3 * (size_t)nx;
  for (int idx = threadIdx.x; idx < nwork * L; idx += blockDim.x) {
    const int w = R.px->dn.div(idx), k = idx - w * L;
    V A = cmk<V>(0, 0), B = cmk<V>(0, 0);
    if (R.rows[w + 1] >= 0) {
      const bool lo = k < hx;
      const int kk = lo ? k : L - k;
      const V* sr = R.specraw + (size_t)w * 3 * hxp;
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
    R.fa[(size_t)(2 * w) * L + k] = A;
    R.fa[(size_t)(2 * w + 1) * L + k] = B;
  }
  __syncthreads();
  V* res = fft_run<T, true>(R.fa, R.fb, 2 * nwork, L, *R.px, R.twx);
  for (int idx = threadIdx.x; idx < nwork * nx; idx += blockDim.x) {
    const int w = R.g.dnx.div(idx), x = idx - w * nx;
    const V a = res[(size_t)(2 * w) * L + x];
    const V b = res[(size_t)(2 * w + 1) * L + x];
    T* hr = R.hsm + (size_t)w * mstride;
    hr[x] = a.x;
    hr[nx + x] = a.y;
    hr[2 * nx + x] = b.x;
  }
  __syncthreads();
}

// colour 0 on the work rows, colour 1 on the band rows; returns this thread's
// accepted trials on band rows
template <typename T>
__device__ __forceinline__ unsigned int row_sweep(const RowPhase<T>& R, const McCoef<T>& c) {
  const int nx = R.g.nx;
  const int nwork = R.nb + 2, half = (nx + 1) >> 1;
  const size_t mstride = 3 * (size_t)nx;
  unsigned int acc = 0;
  for (int color = 0; color < 2; ++color) {
    const int kbase = color == 0 ? 0 : nwork;
    const int kcnt = color == 0 ? nwork : R.nb;
    for (int idx = threadIdx.x; idx < kcnt * half; idx += blockDim.x) {
      const int kq = R.g.dhxc.div(idx);
      const int k = kbase + kq, j = idx - kq * half;
      const int slot = color == 0 ? 1 + k : 2 + (k - nwork);
      const int y = R.rows[slot];
      if (y < 0) continue;
      const int x = 2 * j + ((color + y) & 1);
      if (x >= nx) continue;
      T* row = R.msm + (size_t)slot * mstride;
      Nbrs<T> nbv;
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        int xx = x + (s ? 1 : -1);
        bool ok = true;
        if (xx < 0 || xx >= nx) {
          if (R.g.per[0]) xx = xx < 0 ? xx + nx : xx - nx;
          else ok = false;
        }
        if (xx == x) ok = false;
        nbv.has[0][s] = ok;
        const int xs = ok ? xx : x;
        nbv.v[0][s][0] = row[xs];
        nbv.v[0][s][1] = row[nx + xs];
        nbv.v[0][s][2] = row[2 * nx + xs];
        const int ns = slot + (s ? 1 : -1);
        const bool oky = R.rows[ns] >= 0 && R.rows[ns] != y;
        nbv.has[1][s] = oky;
        const T* r2 = R.msm + (size_t)(oky ? ns : slot) * mstride;
        nbv.v[1][s][0] = r2[x];
        nbv.v[1][s][1] = r2[nx + x];
        nbv.v[1][s][2] = r2[2 * nx + x];
        nbv.has[2][s] = false;
        nbv.v[2][s][0] = nbv.v[2][s][1] = nbv.v[2][s][2] = (T)0;
      }
      const T* hr = R.hsm + (size_t)(slot - 1) * mstride;
      const Proposal<T> p = R.prop[k * half + j];
      if (mc_accept<T>(c, nbv, row[x], row[nx + x], row[2 * nx + x], hr[x], hr[nx + x], hr[2 * nx + x], p)) {
        row[x] = p.x;
        row[nx + x] = p.y;
        row[2 * nx + x] = p.z;
        if (slot >= 2 && slot < 2 + R.nb) acc += 1;
      }
    }
    __syncthreads();
  }
  return acc;
}

// the band's m (and h) back to global memory
template <typename T>
__device__ __forceinline__ void row_store(const RowPhase<T>& R, bool with_h) {
  const int nx = R.g.nx;
  const long long n = R.g.n;
  const size_t mstride = 3 * (size_t)nx;
  const FastDiv dms((uint32_t)mstride);
  for (int idx = threadIdx.x; idx < R.nb * (int)mstride; idx += blockDim.x) {
    const int rr = dms.div(idx), rem = idx - rr * (int)mstride;
    const int cc = R.g.dnx.div(rem), x = rem - cc * nx;
    const long long gi = cc * n + (long long)(R.y0 + rr) * nx + x;
    R.mo[gi] = R.msm[(size_t)(rr + 2) * mstride + rem];
    if (with_h) R.h[gi] = R.hsm[(size_t)(rr + 1) * mstride + rem];
  }
}

// forward x-FFT of the band rows held in msm -> spectrum rows
template <typename T>
__device__ __forceinline__ void row_forward(const RowPhase<T>& R) {
  using V = C<T>;
  const int nx = R.g.nx, hx = R.g.hx, hxp = R.g.hxp, L = R.px->n;
  const long long nspec = R.g.nspec;
  const size_t mstride = 3 * (size_t)nx;
  for (int idx = threadIdx.x; idx < R.nb * L; idx += blockDim.x) {
    const int rr = R.px->dn.div(idx), x = idx - rr * L;
    const T* row = R.msm + (size_t)(rr + 2) * mstride;
    V a = cmk<V>(0, 0), b = cmk<V>(0, 0);
    if (x < nx) {
      a = cmk<V>(row[x], row[nx + x]);
      b = cmk<V>(row[2 * nx + x], (T)0);
    }
    R.fa[(size_t)(2 * rr) * L + x] = a;
    R.fa[(size_t)(2 * rr + 1) * L + x] = b;
  }
  __syncthreads();
  V* res = fft_run<T, false>(R.fa, R.fb, 2 * R.nb, L, *R.px, R.twx);
  for (int idx = threadIdx.x; idx < R.nb * hx; idx += blockDim.x) {
    const int rr = R.g.dhx.div(idx), k = idx - rr * hx;
    const V* la = res + (size_t)(2 * rr) * L;
    const V* lb = la + L;
    const int kn = k == 0 ? 0 : L - k;
    const V A = la[k], B = la[kn];
    const V A2 = lb[k], B2 = lb[kn];
    const long long off = (long long)(R.y0 + rr) * hxp + k;
    R.So[off] = cmk<V>((T)0.5 * (A.x + B.x), (T)0.5 * (A.y - B.y));
    R.So[nspec + off] = cmk<V>((T)0.5 * (A.y + B.y), (T)-0.5 * (A.x - B.x));
    R.So[2 * nspec + off] = cmk<V>((T)0.5 * (A2.x + B2.x), (T)0.5 * (A2.y - B2.y));
  }
}

// Batched row kernel: one CTA per (band, replica).  A batched film sweep is
// this kernel (m, S) -> (mo, So) followed by the column pass on So.
template <typename T>
__global__ void __launch_bounds__(256) k_rows(Geom g, const __grid_constant__ FftPlan px,
                                              const McCoef<T>* __restrict__ coef, const T* m, T* mo, T* h,
                                              const C<T>* S, C<T>* So, unsigned long long* acc,
                                              const SweepCounters* ctr, int band, int with_h, int do_forward) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_rows[64];
  __shared__ unsigned int s_acc;
  const int z = blockIdx.z;
  RowPhase<T> R;
  R.g = g;
  R.px = &px;
  const bool two_fft = px.warp_a == 0;
  unsigned char* ptr = smem_raw;
  row_phase_carve<T>(R, ptr, band, two_fft);
  R.rows = s_rows;
  R.m = m + (long long)z * 3 * g.n;
  R.mo = mo + (long long)z * 3 * g.n;
  R.h = h + (long long)z * 3 * g.n;
  R.S = S + (long long)z * 3 * g.nspec;
  R.So = So + (long long)z * 3 * g.nspec;
  R.y0 = blockIdx.x * band;
  R.nb = max(0, min(band, g.ny - R.y0));
  const McCoef<T> c = coef[z];
  if (threadIdx.x < R.nb + 4) s_rows[threadIdx.x] = band_row(R.y0 - 2 + (int)threadIdx.x, g.ny, g.per[1]);
  if (threadIdx.x == 0) s_acc = 0;
  load_twiddles<T>(px, R.twx);
  __syncthreads();
  row_load<T>(R, c, ctr->stage, ctr->sweep);
  row_field<T>(R);
  unsigned int a = row_sweep<T>(R, c);
  row_store<T>(R, with_h != 0);
  if (do_forward) row_forward<T>(R);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
  if ((threadIdx.x & 31) == 0 && a) atomicAdd(&s_acc, a);
  __syncthreads();
  if (threadIdx.x == 0 && s_acc) atomicAdd(acc + z, (unsigned long long)s_acc);
}

}  // namespace mmc
