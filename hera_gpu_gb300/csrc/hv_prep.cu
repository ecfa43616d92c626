// hv_prep.cu -- per-call and per-time preparation kernels.
//
//  * beam transpose: the reference uploads bm_cube into a 3-D texture
//    (hera_gpu/vis.py:113-138, 198); here the beam stays in global memory as
//    [pixel][antenna] so that a warp whose lanes are antennas gathers one
//    128-byte line per beam corner.
//  * phase coefficients: the reference forms tau = antpos . (eq2top . crd_eq)
//    / c with two GEMMs per chunk (vis.py:230-235) and multiplies by 2 pi nu
//    in MeasEq (vis.py:107).  Since p . (R s) = (R^T p) . s, the per-antenna
//    vector U = nu / c * R^T p is formed once per (time, frequency) in FP64
//    and the phase in cycles is U . s_eq.
//  * source prep: rotation to topocentric, horizon cut (vis.py:75, 85-86) and
//    the bilinear corner / weights (vis.py:63-73), once per time and shared
//    by every antenna and frequency.  Sources below the horizon are dropped
//    (the reference computes them and multiplies by A = 0); the survivors keep
//    their input order, so the split-K order is deterministic.
#include <algorithm>

#include "hv_internal.cuh"
#include "hv_kernels.h"

namespace hv {

// ---------------------------------------------------------------- beam ----
template <typename R>
__global__ void beam_transpose_kernel(const R* __restrict__ bm, int nant, int PP, int Np,
                                      R* __restrict__ beamT) {
  __shared__ R tile[32][33];
  const int f = blockIdx.z;
  const int pix0 = blockIdx.x * 32, a0 = blockIdx.y * 32;
  const R* src = bm + (size_t)f * nant * PP;
  R* dst = beamT + (size_t)f * PP * Np;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int a = a0 + j, pix = pix0 + threadIdx.x;
    tile[j][threadIdx.x] = (a < nant && pix < PP) ? src[(size_t)a * PP + pix] : R(0);
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int pix = pix0 + j, a = a0 + threadIdx.x;
    if (pix < PP && a < Np) dst[(size_t)pix * Np + a] = tile[threadIdx.x][j];
  }
}

template <typename R>
cudaError_t launch_beam_transpose(const R* bm, int nfreq, int nant, int P, int Np,
                                  R* beamT, cudaStream_t st) {
  const int PP = P * P;
  dim3 grid(ceil_div(PP, 32), Np / 32, nfreq), block(32, 8);
  beam_transpose_kernel<R><<<grid, block, 0, st>>>(bm, nant, PP, Np, beamT);
  return cudaGetLastError();
}

// ----------------------------------------------------------- U coeffs ----
__device__ __forceinline__ void store_ucoef(Ucoef32* U, size_t i, const double u[3]) {
  Ucoef32 c;
  c.hx = (float)u[0]; c.hy = (float)u[1]; c.hz = (float)u[2]; c.p0 = 0.f;
  c.lx = (float)(u[0] - (double)c.hx);
  c.ly = (float)(u[1] - (double)c.hy);
  c.lz = (float)(u[2] - (double)c.hz);
  c.p1 = 0.f;
  U[i] = c;
}
__device__ __forceinline__ void store_ucoef(Ucoef64* U, size_t i, const double u[3]) {
  Ucoef64 c;
  c.x = u[0]; c.y = u[1]; c.z = u[2]; c.p = 0.0;
  U[i] = c;
}

template <typename R>
__global__ void ucoef_kernel(const R* __restrict__ antpos, int nant, int Np,
                             const R* __restrict__ eq2tops, int t0, int nt,
                             const double* __restrict__ freqs, int nfreq,
                             typename Traits<R>::U* __restrict__ U) {
  const size_t total = (size_t)nt * nfreq * Np;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int a = (int)(i % Np);
    const int f = (int)((i / Np) % nfreq);
    const int tt = (int)(i / ((size_t)Np * nfreq));
    double u[3] = {0.0, 0.0, 0.0};
    if (a < nant) {
      const R* M = eq2tops + (size_t)(t0 + tt) * 9;
      const double p0 = antpos[a * 3 + 0], p1 = antpos[a * 3 + 1], p2 = antpos[a * 3 + 2];
      const double scale = freqs[f] / kSpeedOfLight;
      for (int k = 0; k < 3; ++k) {
        // (R^T p)_k = sum_j R[j][k] p_j
        const double w = fma((double)M[0 * 3 + k], p0,
                             fma((double)M[1 * 3 + k], p1, (double)M[2 * 3 + k] * p2));
        u[k] = w * scale;
      }
    }
    store_ucoef(U, i, u);
  }
}

template <typename R>
cudaError_t launch_ucoef(const R* antpos, int nant, int Np, const R* eq2tops, int t0,
                         int nt, const double* d_freqs, int nfreq, void* U,
                         cudaStream_t st) {
  const size_t total = (size_t)nt * nfreq * Np;
  const int blocks = (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
  ucoef_kernel<R><<<blocks > 0 ? blocks : 1, 256, 0, st>>>(
      antpos, nant, Np, eq2tops, t0, nt, d_freqs, nfreq,
      reinterpret_cast<typename Traits<R>::U*>(U));
  return cudaGetLastError();
}

__global__ void __launch_bounds__(256)
ubound_kernel(const Ucoef32* __restrict__ U, int Np, float* __restrict__ umax) {
  __shared__ float red[8];
  const Ucoef32* u = U + (size_t)blockIdx.x * Np;
  float m = 0.f;
  for (int a = threadIdx.x; a < Np; a += blockDim.x) {
    const Ucoef32 c = u[a];
    m = fmaxf(m, fabsf(c.hx) + fabsf(c.hy) + fabsf(c.hz));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < 8; ++w) m = fmaxf(m, red[w]);
    umax[blockIdx.x] = m * 1.0001f;  // margin for the rounding of the sum
  }
}

cudaError_t launch_ubound(const void* U, int nslices, int Np, float* umax, cudaStream_t st) {
  ubound_kernel<<<nslices, 256, 0, st>>>(static_cast<const Ucoef32*>(U), Np, umax);
  return cudaGetLastError();
}

// -------------------------------------------------------- source prep ----
int prep_blocks(int nsrc) { return nsrc > 0 ? ceil_div(nsrc, kPrepBlock) : 1; }

template <typename R>
__device__ __forceinline__ void load_rot(const R* __restrict__ eq2tops, int t, double* rot) {
  if (threadIdx.x < 9) rot[threadIdx.x] = (double)eq2tops[(size_t)t * 9 + threadIdx.x];
}

// z component of eq2top . s (topocentric up), FP64.
__device__ __forceinline__ double top_z(const double* rot, double x, double y, double z) {
  return fma(rot[6], x, fma(rot[7], y, rot[8] * z));
}

template <typename R>
__global__ void __launch_bounds__(kPrepBlock)
prep_count_kernel(const R* __restrict__ crd_eq, int nsrc, const R* __restrict__ eq2tops,
                  int t0, int nblk, int* __restrict__ block_counts) {
  __shared__ double rot[9];
  __shared__ int warp_cnt[kPrepBlock / 32];
  const int tt = blockIdx.y;
  load_rot(eq2tops, t0 + tt, rot);
  __syncthreads();
  const int s = blockIdx.x * kPrepBlock + threadIdx.x;
  bool up = false;
  if (s < nsrc)
    up = top_z(rot, crd_eq[s], crd_eq[(size_t)nsrc + s], crd_eq[2 * (size_t)nsrc + s]) > 0.0;
  const unsigned m = __ballot_sync(0xffffffffu, up);
  if ((threadIdx.x & 31) == 0) warp_cnt[threadIdx.x >> 5] = __popc(m);
  __syncthreads();
  if (threadIdx.x < 32) {
    int c = warp_cnt[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (threadIdx.x == 0) block_counts[(size_t)tt * nblk + blockIdx.x] = c;
  }
}

__device__ __forceinline__ void fill_rec(SrcRec32& r, double x, double y, double z,
                                         double amp, int pix, double fx, double fy) {
  r.sx = (float)x; r.sy = (float)y; r.sz = (float)z; r.amp = (float)amp;
  r.pix = pix; r.fx = (float)fx; r.fy = (float)fy; r.pad = 0;
}
__device__ __forceinline__ void fill_rec(SrcRec64& r, double x, double y, double z,
                                         double amp, int pix, double fx, double fy) {
  r.sx = x; r.sy = y; r.sz = z; r.amp = amp; r.fx = fx; r.fy = fy; r.pix = pix;
  r.pad[0] = r.pad[1] = r.pad[2] = 0;
}

// Lower corner and weight along one beam axis, clamped so that the four
// gathered texels always lie inside the P x P grid.  Outside the grid the
// value is the edge texel's, as with the reference's clamped texture
// (vis.py:39) and RectBivariateSpline (test_vis_gpu.py:334).
__device__ __forceinline__ int beam_axis(double c, int P, double& w) {
  const double b = (P - 1) * fma(0.5, c, 0.5);
  const double fb = floor(b);
  w = b - fb;
  if (P < 2) { w = 0.0; return 0; }
  if (fb < 0.0) w = 0.0;
  if (fb >= (double)(P - 1)) w = 1.0;
  return (int)fmin(fmax(fb, 0.0), (double)(P - 2));
}

template <typename R>
__global__ void __launch_bounds__(kPrepBlock)
prep_write_kernel(const R* __restrict__ crd_eq, const R* __restrict__ I_sky, int nsrc,
                  size_t rec_stride, const R* __restrict__ eq2tops, int t0, int nblk, int P,
                  const int* __restrict__ block_counts,
                  typename Traits<R>::Rec* __restrict__ rec, int* __restrict__ count) {
  __shared__ double rot[9];
  __shared__ int warp_cnt[kPrepBlock / 32];
  __shared__ int red[kPrepBlock / 32];
  __shared__ int base;
  const int tt = blockIdx.y;
  const int* bc = block_counts + (size_t)tt * nblk;
  load_rot(eq2tops, t0 + tt, rot);
  // offset of this block = sum of the counts of the blocks before it
  int part = 0;
  for (int i = threadIdx.x; i < (int)blockIdx.x; i += kPrepBlock) part += bc[i];
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x < 32) {
    int c = red[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (threadIdx.x == 0) base = c;
  }
  const int s = blockIdx.x * kPrepBlock + threadIdx.x;
  double x = 0, y = 0, z = 0, tx = 0, ty = 0, tz = 0;
  bool up = false;
  __syncthreads();
  if (s < nsrc) {
    x = crd_eq[s]; y = crd_eq[(size_t)nsrc + s]; z = crd_eq[2 * (size_t)nsrc + s];
    tx = fma(rot[0], x, fma(rot[1], y, rot[2] * z));
    ty = fma(rot[3], x, fma(rot[4], y, rot[5] * z));
    tz = top_z(rot, x, y, z);
    up = tz > 0.0;
  }
  const unsigned m = __ballot_sync(0xffffffffu, up);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) warp_cnt[warp] = __popc(m);
  __syncthreads();
  if (warp == 0) {  // exclusive scan of the warp counts
    const int c = warp_cnt[lane];
    int incl = c;
    for (int o = 1; o < 32; o <<= 1) {
      const int n = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += n;
    }
    red[lane] = incl - c;
    if (blockIdx.x == nblk - 1 && lane == 31) count[tt] = base + incl;
  }
  __syncthreads();
  if (up) {
    const int idx = base + red[warp] + __popc(m & ((1u << lane) - 1u));
    double fx, fy;
    const int px = beam_axis(tx, P, fx);
    const int py = beam_axis(ty, P, fy);
    typename Traits<R>::Rec r;
    fill_rec(r, x, y, z, sqrt((double)I_sky[s]), py * P + px, fx, fy);
    rec[(size_t)tt * rec_stride + idx] = r;
  }
}

template <typename R>
cudaError_t launch_prep_strided(const R* crd_eq, const R* I_sky, int nsrc, const R* eq2tops,
                                int t0, int nt, int P, int* block_counts, void* rec,
                                size_t rec_stride, int* count, cudaStream_t st) {
  const int nblk = prep_blocks(nsrc);
  dim3 grid(nblk, nt);
  prep_count_kernel<R><<<grid, kPrepBlock, 0, st>>>(crd_eq, nsrc, eq2tops, t0, nblk,
                                                    block_counts);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  prep_write_kernel<R><<<grid, kPrepBlock, 0, st>>>(
      crd_eq, I_sky, nsrc, rec_stride, eq2tops, t0, nblk, P, block_counts,
      reinterpret_cast<typename Traits<R>::Rec*>(rec), count);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_prep(const R* crd_eq, const R* I_sky, int nsrc, const R* eq2tops,
                        int t0, int nt, int P, int* block_counts, void* rec,
                        int* count, cudaStream_t st) {
  return launch_prep_strided<R>(crd_eq, I_sky, nsrc, eq2tops, t0, nt, P, block_counts, rec,
                                (size_t)nsrc, count, st);
}

// ---------------------------------------------------- fused-path records --
// Prepares the records of each time for the fused kernel, in place:
//  * record 0 of each unit of 8 consecutive records (the 8 sources one
//    generator thread handles together) gets, in its pad word, the largest
//    |s - s_ref|_1 over the unit (s_ref = record 0's direction), with the
//    sign bit set if all eight share record 0's beam pixel: the fused kernel
//    takes phases relative to s_ref when the spread is small enough for the
//    slice at hand, and loads the four beam corners once for such a unit;
//  * records [count, round_up(count, 32)) are zeroed, so a partial last stage
//    reads sources of zero amplitude at beam pixel 0.
__global__ void __launch_bounds__(256)
tc_relative_kernel(SrcRec32* __restrict__ rec, size_t rec_stride,
                   const int* __restrict__ counts) {
  const int tt = blockIdx.y;
  SrcRec32* r = rec + (size_t)tt * rec_stride;
  const int n = counts[tt];
  const int npad = (n + 31) & ~31;
  for (int i0 = blockIdx.x * blockDim.x; i0 < npad; i0 += gridDim.x * blockDim.x) {
    const int i = i0 + threadIdx.x;  // a warp covers 4 whole units
    float d1 = 0.f;
    int pix = -1, ref_pix = -1;
    if (i < n) {
      const SrcRec32 ref = r[i & ~7];
      const SrcRec32 me = r[i];
      d1 = fabsf(me.sx - ref.sx) + fabsf(me.sy - ref.sy) + fabsf(me.sz - ref.sz);
      pix = me.pix;
      ref_pix = ref.pix;
    }
    // over the 8 lanes of the unit: largest spread, and whether every
    // source sits on the reference's beam pixel (padding counts as same)
    for (int o = 4; o > 0; o >>= 1) d1 = fmaxf(d1, __shfl_xor_sync(0xffffffffu, d1, o));
    const unsigned differ = __ballot_sync(0xffffffffu, i < n && pix != ref_pix);
    const bool same_pix = ((differ >> (threadIdx.x & 24)) & 0xffu) == 0;
    __syncwarp();
    if (i < n) {
      // pad word of the unit's first record: the spread as a float, with the
      // sign bit set when all eight sources share one beam pixel
      if ((i & 7) == 0) r[i].pad = __float_as_int(d1) | (same_pix ? (int)0x80000000u : 0);
    } else if (i < npad) {
      r[i] = SrcRec32{};
    }
  }
}

cudaError_t launch_tc_relative(void* rec, size_t rec_stride, const int* counts, int nt, int nsrc,
                               cudaStream_t st) {
  const int blocks = std::max(1, std::min(ceil_div(nsrc, 256), 2048));
  dim3 grid(blocks, nt);
  tc_relative_kernel<<<grid, 256, 0, st>>>(static_cast<SrcRec32*>(rec), rec_stride, counts);
  return cudaGetLastError();
}

// ---------------------------------------- FP16 + FP8 form: slice bounds --
// pixmax[f][pix] = max over antennas of |beamT[f][pix][a]|: one warp per
// (frequency, pixel) row of the transposed beam.
__global__ void __launch_bounds__(256)
beam_pixmax_kernel(const float* __restrict__ beamT, long long rows, int Np,
                   float* __restrict__ pixmax) {
  const int lane = threadIdx.x & 31;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += nw) {
    const float* row = beamT + r * Np;
    float m = 0.f;
    for (int a = lane; a < Np; a += 32) m = fmaxf(m, fabsf(row[a]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) pixmax[r] = m;
  }
}

cudaError_t launch_beam_pixmax(const float* beamT, int nfreq, int P, int Np, float* pixmax,
                               cudaStream_t st) {
  const long long rows = (long long)nfreq * P * P;
  const long long blocks = std::min<long long>(4096, (rows + 7) / 8);
  beam_pixmax_kernel<<<(int)std::max<long long>(blocks, 1), 256, 0, st>>>(beamT, rows, Np,
                                                                          pixmax);
  return cudaGetLastError();
}

// sbound[tt][f] = max over the records of time tt of sqrt(I) x the largest
// |beam| over antennas at the record's four beam corners: a bound of |A|
// sqrt(I) over the slice (bilinear weights lie in [0, 1]).  Each thread
// holds up to kBoundRecs records; per frequency a warp reduces and one lane
// raises the slice's bound (float bits of non-negative values order as
// unsigned integers).  sbound must be zero beforehand.
constexpr int kBoundRecs = 4;
__global__ void __launch_bounds__(256)
slice_bound_kernel(const SrcRec32* __restrict__ rec, size_t rec_stride,
                   const int* __restrict__ counts, const float* __restrict__ pixmax, int nf,
                   int PP, int dx, int dy, unsigned* __restrict__ sbound) {
  const int tt = blockIdx.y;
  const int n = counts[tt];
  const SrcRec32* r = rec + (size_t)tt * rec_stride;
  for (long long base = (long long)blockIdx.x * blockDim.x * kBoundRecs; base < n;
       base += (long long)gridDim.x * blockDim.x * kBoundRecs) {
    int pix[kBoundRecs];
    float amp[kBoundRecs];
#pragma unroll
    for (int k = 0; k < kBoundRecs; ++k) {
      const long long i = base + (long long)k * blockDim.x + threadIdx.x;
      pix[k] = 0;
      amp[k] = 0.f;
      if (i < n) {
        pix[k] = r[i].pix;
        amp[k] = fabsf(r[i].amp);
      }
    }
    for (int f = 0; f < nf; ++f) {
      const float* pm = pixmax + (size_t)f * PP;
      float m = 0.f;
#pragma unroll
      for (int k = 0; k < kBoundRecs; ++k) {
        if (amp[k] == 0.f) continue;
        const int q = pix[k];
        const float c = fmaxf(fmaxf(__ldg(pm + q), __ldg(pm + q + dx)),
                              fmaxf(__ldg(pm + q + dy), __ldg(pm + q + dx + dy)));
        m = fmaxf(m, amp[k] * c);
      }
      for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
      if ((threadIdx.x & 31) == 0 && m > 0.f)
        atomicMax(sbound + (size_t)tt * nf + f, __float_as_uint(m));
    }
  }
}

cudaError_t launch_slice_bound(const void* rec, size_t rec_stride, const int* counts, int nt,
                               int nsrc, const float* pixmax, int nf, int P, float* sbound,
                               cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(sbound, 0, sizeof(float) * (size_t)nt * nf, st);
  if (e != cudaSuccess) return e;
  const int per_block = 256 * kBoundRecs;
  const int blocks = std::max(1, std::min(ceil_div(std::max(nsrc, 1), per_block), 1024));
  dim3 grid(blocks, nt);
  slice_bound_kernel<<<grid, 256, 0, st>>>(static_cast<const SrcRec32*>(rec), rec_stride, counts,
                                           pixmax, nf, P * P, P > 1 ? 1 : 0, P > 1 ? P : 0,
                                           reinterpret_cast<unsigned*>(sbound));
  return cudaGetLastError();
}

template cudaError_t launch_beam_transpose<float>(const float*, int, int, int, int, float*, cudaStream_t);
template cudaError_t launch_beam_transpose<double>(const double*, int, int, int, int, double*, cudaStream_t);
template cudaError_t launch_ucoef<float>(const float*, int, int, const float*, int, int, const double*, int, void*, cudaStream_t);
template cudaError_t launch_ucoef<double>(const double*, int, int, const double*, int, int, const double*, int, void*, cudaStream_t);
template cudaError_t launch_prep<float>(const float*, const float*, int, const float*, int, int, int, int*, void*, int*, cudaStream_t);
template cudaError_t launch_prep_strided<float>(const float*, const float*, int, const float*, int, int, int, int*, void*, size_t, int*, cudaStream_t);
template cudaError_t launch_prep<double>(const double*, const double*, int, const double*, int, int, int, int*, void*, int*, cudaStream_t);

}  // namespace hv
