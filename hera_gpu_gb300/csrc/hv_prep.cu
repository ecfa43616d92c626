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
#include <type_traits>

#include "hv_internal.cuh"
#include "hv_kernels.h"

namespace hv {

// ---------------------------------------------------------------- beam ----
// One 32 x 32 (pixel, antenna) tile of frequency f (block 32 x 8 threads).
template <typename R>
__device__ __forceinline__ void beam_transpose_tile(const R* __restrict__ bm, int nant, int PP,
                                                    int Np, R* __restrict__ beamT, int f,
                                                    int pix0, int a0, R (*tile)[33]) {
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
__global__ void beam_transpose_kernel(const R* __restrict__ bm, int nant, int PP, int Np,
                                      R* __restrict__ beamT) {
  __shared__ R tile[32][33];
  beam_transpose_tile<R>(bm, nant, PP, Np, beamT, blockIdx.z, blockIdx.x * 32, blockIdx.y * 32,
                         tile);
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

// Element i = (tt * nfreq + f) * Np + a of U.
template <typename R>
__device__ __forceinline__ void ucoef_element(const R* __restrict__ antpos, int nant, int Np,
                                              const R* __restrict__ eq2tops, int t0,
                                              const double* __restrict__ freqs, int nfreq,
                                              typename Traits<R>::U* __restrict__ U, size_t i) {
  {
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
__global__ void ucoef_kernel(const R* __restrict__ antpos, int nant, int Np,
                             const R* __restrict__ eq2tops, int t0, int nt,
                             const double* __restrict__ freqs, int nfreq,
                             typename Traits<R>::U* __restrict__ U) {
  const size_t total = (size_t)nt * nfreq * Np;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x)
    ucoef_element<R>(antpos, nant, Np, eq2tops, t0, freqs, nfreq, U, i);
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

// Bound of one slice (block of 256 threads).
__device__ __forceinline__ void ubound_slice(const Ucoef32* __restrict__ u, int Np,
                                             float* __restrict__ out, float* red) {
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
    *out = m * 1.0001f;  // margin for the rounding of the sum
  }
}

__global__ void __launch_bounds__(256)
ubound_kernel(const Ucoef32* __restrict__ U, int Np, float* __restrict__ umax) {
  __shared__ float red[8];
  ubound_slice(U + (size_t)blockIdx.x * Np, Np, umax + blockIdx.x, red);
}

cudaError_t launch_ubound(const void* U, int nslices, int Np, float* umax, cudaStream_t st) {
  ubound_kernel<<<nslices, 256, 0, st>>>(static_cast<const Ucoef32*>(U), Np, umax);
  return cudaGetLastError();
}

// -------------------------------------------------------- source prep ----
__host__ __device__ int prep_blocks_of(int nsrc) { return nsrc > 0 ? ceil_div(nsrc, kPrepBlock) : 1; }
int prep_blocks(int nsrc) { return prep_blocks_of(nsrc); }

template <typename R>
__device__ __forceinline__ void load_rot(const R* __restrict__ eq2tops, int t, R* rot) {
  if (threadIdx.x < 9) rot[threadIdx.x] = eq2tops[(size_t)t * 9 + threadIdx.x];
}

// Topocentric geometry of one source at one time: the horizon test on the
// z component of eq2top . s, and the beam corner and weights from its x
// and y components.
//
// FP32 inputs: each component is formed as an unevaluated sum hi + lo with
// error-free transformations (TwoProduct by FMA, TwoSum; the compensated dot
// product Dot2 of Ogita, Rump and Oishi, "Accurate sum and dot product",
// SIAM J. Sci. Comput. 26(6), 2005), whose error is at most
// u |r . s| + gamma_3^2 sum |r_i s_i| (u = 2^-24): the horizon test and the
// weights come out as they would from an FP64 evaluation, in FP32
// arithmetic (this part's FP64 rate is a small fraction of its FP32 rate,
// and the work is per source and time).  FP64 inputs use FP64.
struct FF {
  float hi, lo;
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bv = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bv)), __fsub_rn(b, bv));
}

__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}

// r[0] x + r[1] y + r[2] z as hi + lo (hi = the sum rounded once).
__device__ __forceinline__ FF dot3(const float* r, float x, float y, float z) {
  float p, s, h, e, q;
  two_prod(r[0], x, p, s);
  two_prod(r[1], y, h, e);
  two_sum(p, h, p, q);
  s = __fadd_rn(s, __fadd_rn(q, e));
  two_prod(r[2], z, h, e);
  two_sum(p, h, p, q);
  s = __fadd_rn(s, __fadd_rn(q, e));
  FF out;
  two_sum(p, s, out.hi, out.lo);
  return out;
}

// Above the horizon: topocentric z > 0 (hi has the sign of hi + lo).
__device__ __forceinline__ bool above_horizon(const float* rot, float x, float y, float z) {
  return dot3(rot + 6, x, y, z).hi > 0.f;
}
__device__ __forceinline__ bool above_horizon(const double* rot, double x, double y, double z) {
  return fma(rot[6], x, fma(rot[7], y, rot[8] * z)) > 0.0;
}

// Source block bx of time tt: sources above the horizon, into
// block_counts[tt * nblk + bx].
template <typename R>
__device__ __forceinline__ void prep_count_block(const R* __restrict__ crd_eq, int nsrc,
                                                 const R* __restrict__ eq2tops, int t0, int nblk,
                                                 int* __restrict__ block_counts, int bx, int tt,
                                                 R* rot, int* warp_cnt) {
  load_rot(eq2tops, t0 + tt, rot);
  __syncthreads();
  const int s = bx * kPrepBlock + threadIdx.x;
  bool up = false;
  if (s < nsrc)
    up = above_horizon(rot, crd_eq[s], crd_eq[(size_t)nsrc + s], crd_eq[2 * (size_t)nsrc + s]);
  const unsigned m = __ballot_sync(0xffffffffu, up);
  if ((threadIdx.x & 31) == 0) warp_cnt[threadIdx.x >> 5] = __popc(m);
  __syncthreads();
  if (threadIdx.x < 32) {
    int c = warp_cnt[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (threadIdx.x == 0) block_counts[(size_t)tt * nblk + bx] = c;
  }
}

template <typename R>
__global__ void __launch_bounds__(kPrepBlock)
prep_count_kernel(const R* __restrict__ crd_eq, int nsrc, const R* __restrict__ eq2tops,
                  int t0, int nblk, int* __restrict__ block_counts) {
  __shared__ R rot[9];
  __shared__ int warp_cnt[kPrepBlock / 32];
  prep_count_block<R>(crd_eq, nsrc, eq2tops, t0, nblk, block_counts, blockIdx.x, blockIdx.y, rot,
                      warp_cnt);
}

// Lower corner and weight along one beam axis, clamped so that the four
// gathered texels always lie inside the P x P grid.  Outside the grid the
// value is the edge texel's, as with the reference's clamped texture
// (vis.py:39) and RectBivariateSpline (test_vis_gpu.py:334).  The texel
// coordinate is b = (P - 1)(c / 2 + 1 / 2) (vis.py:63-73).
__device__ __forceinline__ int beam_axis(double c, int P, double& w) {
  const double b = (P - 1) * fma(0.5, c, 0.5);
  const double fb = floor(b);
  w = b - fb;
  if (P < 2) { w = 0.0; return 0; }
  if (fb < 0.0) w = 0.0;
  if (fb >= (double)(P - 1)) w = 1.0;
  return (int)fmin(fmax(fb, 0.0), (double)(P - 2));
}

// The same from c = hi + lo in FP32: b = h (c + 1), h = (P - 1) / 2 (exact),
// carried as b + be; b - floor(b) is exact, and the weight is rounded once.
__device__ __forceinline__ int beam_axis(FF c, int P, float& w) {
  const float h = 0.5f * (float)(P - 1);
  float u, ue, b, be;
  two_sum(c.hi, 1.f, u, ue);
  ue = __fadd_rn(ue, c.lo);
  two_prod(h, u, b, be);
  be = __fmaf_rn(h, ue, be);
  float fb = floorf(b);
  float f = __fadd_rn(__fsub_rn(b, fb), be);
  if (f < 0.f) {  // b + be lies just below the integer b
    fb -= 1.f;
    f = __fadd_rn(f, 1.f);
  } else if (f >= 1.f) {
    fb += 1.f;
    f = __fsub_rn(f, 1.f);
  }
  w = f;
  if (P < 2) { w = 0.f; return 0; }
  if (fb < 0.f) w = 0.f;
  if (fb >= (float)(P - 1)) w = 1.f;
  return (int)fminf(fmaxf(fb, 0.f), (float)(P - 2));
}

// The record of a source above the horizon: its direction, sqrt(I) (sqrtf
// is correctly rounded, as is the FP64 square root rounded to FP32), and
// its beam corner and weights.
__device__ __forceinline__ void fill_rec(SrcRec32& r, const float* rot, float x, float y,
                                         float z, float I, int P) {
  float fx, fy;
  const int px = beam_axis(dot3(rot, x, y, z), P, fx);
  const int py = beam_axis(dot3(rot + 3, x, y, z), P, fy);
  r.sx = x; r.sy = y; r.sz = z; r.amp = sqrtf(I);
  r.pix = py * P + px; r.fx = fx; r.fy = fy; r.pad = 0;
}
__device__ __forceinline__ void fill_rec(SrcRec64& r, const double* rot, double x, double y,
                                         double z, double I, int P) {
  double fx, fy;
  const int px = beam_axis(fma(rot[0], x, fma(rot[1], y, rot[2] * z)), P, fx);
  const int py = beam_axis(fma(rot[3], x, fma(rot[4], y, rot[5] * z)), P, fy);
  r.sx = x; r.sy = y; r.sz = z; r.amp = sqrt(I); r.fx = fx; r.fy = fy; r.pix = py * P + px;
  r.pad[0] = r.pad[1] = r.pad[2] = 0;
}

// Ascending bitonic sort of the first n keys of a block (n a power of two,
// 32 <= n <= blockDim.x, the same in every thread): thread i < n returns the
// i-th smallest; the others return their v.  Exchanges at distance >= 32 go
// through sk, shorter ones through warp shuffles.
__device__ __forceinline__ uint32_t block_sort(uint32_t v, uint32_t* sk, int n) {
  const int i = threadIdx.x;
  const bool act = i < n;
#pragma unroll 1
  for (int k = 2; k <= n; k <<= 1) {
#pragma unroll 1
    for (int j = k >> 1; j > 0; j >>= 1) {
      uint32_t o;
      if (j >= 32) {
        if (act) sk[i] = v;
        __syncthreads();
        o = act ? sk[i ^ j] : v;
        __syncthreads();
      } else {
        o = __shfl_xor_sync(0xffffffffu, v, j);
      }
      // the lower index of a pair keeps the minimum when the pair sorts
      // ascending ((i & k) == 0), the maximum otherwise
      const bool keep_min = ((i & j) == 0) == ((i & k) == 0);
      if (act) v = keep_min ? min(v, o) : max(v, o);
    }
  }
  return v;
}

static_assert(kPrepBlock <= 1024, "a key holds 10 bits of index within the block");
// Beams up to this size are written in pixel order (a key holds the pixel in
// its upper 22 bits).
constexpr int kPixelOrderMaxP = 2048;

// FP32 records pass through shared memory so that a block writes them in
// beam-pixel order (sources of one pixel in catalogue order).
template <typename R>
struct PrepOrder {};
template <>
struct PrepOrder<float> {
  uint32_t key[kPrepBlock];
  SrcRec32 rec[kPrepBlock];
};

// Source block bx of time tt: records of its sources above the horizon, at
// the block's place in the time's list (after the blocks before it).  FP32
// records of beams up to kPixelOrderMaxP pixels a side are written in
// beam-pixel order within the block (ties in catalogue order): the
// catalogue is in spatial order, so a block covers a few neighbouring beam
// pixels, and in pixel order most units of 8 consecutive records share one
// pixel (the fused kernel then loads that pixel's four corners once per
// unit).  Other records keep catalogue order.
template <typename R>
struct PrepWriteSmem {
  R rot[9];
  int warp_cnt[kPrepBlock / 32];
  int red[kPrepBlock / 32];
  int base, total;
  PrepOrder<R> ord;
};
template <typename R>
__device__ __forceinline__ void prep_write_block(const R* __restrict__ crd_eq,
                                                 const R* __restrict__ I_sky, int nsrc,
                                                 size_t rec_stride, const R* __restrict__ eq2tops,
                                                 int t0, int nblk, int P,
                                                 const int* __restrict__ block_counts,
                                                 typename Traits<R>::Rec* __restrict__ rec,
                                                 int* __restrict__ count, int bx, int tt,
                                                 PrepWriteSmem<R>& sm) {
  R* rot = sm.rot;
  int* warp_cnt = sm.warp_cnt;
  int* red = sm.red;
  int& base = sm.base;
  const int* bc = block_counts + (size_t)tt * nblk;
  load_rot(eq2tops, t0 + tt, rot);
  // offset of this block = sum of the counts of the blocks before it
  int part = 0;
  for (int i = threadIdx.x; i < bx; i += kPrepBlock) part += bc[i];
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x < 32) {
    int c = red[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (threadIdx.x == 0) base = c;
  }
  const int s = bx * kPrepBlock + threadIdx.x;
  R x = 0, y = 0, z = 0;
  bool up = false;
  __syncthreads();
  if (s < nsrc) {
    x = crd_eq[s]; y = crd_eq[(size_t)nsrc + s]; z = crd_eq[2 * (size_t)nsrc + s];
    up = above_horizon(rot, x, y, z);
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
    if (lane == 31) sm.total = incl;
    if (bx == nblk - 1 && lane == 31) count[tt] = base + incl;
  }
  __syncthreads();
  if constexpr (std::is_same<R, float>::value) {
    if (P <= kPixelOrderMaxP) {
      // the block's records and keys (pixel, catalogue rank), compacted
      const int total = sm.total;
      if (up) {
        const int c = red[warp] + __popc(m & ((1u << lane) - 1u));
        SrcRec32 r;
        fill_rec(r, rot, x, y, z, I_sky[s], P);
        sm.ord.rec[c] = r;
        sm.ord.key[c] = ((uint32_t)r.pix << 10) | (uint32_t)c;
      }
      __syncthreads();
      int n = 32;
      while (n < total) n <<= 1;
      uint32_t key = (int)threadIdx.x < total ? sm.ord.key[threadIdx.x] : 0xffffffffu;
      key = block_sort(key, sm.ord.key, n);
      if ((int)threadIdx.x < total)
        rec[(size_t)tt * rec_stride + base + threadIdx.x] = sm.ord.rec[key & (kPrepBlock - 1)];
      return;
    }
  }
  if (up) {
    const int idx = base + red[warp] + __popc(m & ((1u << lane) - 1u));
    typename Traits<R>::Rec r;
    fill_rec(r, rot, x, y, z, I_sky[s], P);
    rec[(size_t)tt * rec_stride + idx] = r;
  }
}

template <typename R>
__global__ void __launch_bounds__(kPrepBlock)
prep_write_kernel(const R* __restrict__ crd_eq, const R* __restrict__ I_sky, int nsrc,
                  size_t rec_stride, const R* __restrict__ eq2tops, int t0, int nblk, int P,
                  const int* __restrict__ block_counts,
                  typename Traits<R>::Rec* __restrict__ rec, int* __restrict__ count) {
  __shared__ PrepWriteSmem<R> sm;
  prep_write_block<R>(crd_eq, I_sky, nsrc, rec_stride, eq2tops, t0, nblk, P, block_counts, rec,
                      count, blockIdx.x, blockIdx.y, sm);
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
// Records [i0, i0 + 256) of time tt (block of 256 threads).
__device__ __forceinline__ void tc_relative_span(SrcRec32* __restrict__ rec, size_t rec_stride,
                                                 const int* __restrict__ counts, int tt, int i0) {
  SrcRec32* r = rec + (size_t)tt * rec_stride;
  const int n = counts[tt];
  const int npad = (n + 31) & ~31;
  if (i0 >= npad) return;
  {
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

__global__ void __launch_bounds__(256)
tc_relative_kernel(SrcRec32* __restrict__ rec, size_t rec_stride,
                   const int* __restrict__ counts) {
  const int tt = blockIdx.y;
  const int npad = (counts[tt] + 31) & ~31;
  for (int i0 = blockIdx.x * blockDim.x; i0 < npad; i0 += gridDim.x * blockDim.x)
    tc_relative_span(rec, rec_stride, counts, tt, i0);
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

// ------------------------------------------------------------ batches ----
// The same preparation for every simulation of a batch in one launch per
// step; a block finds its simulation in the step's prefix table.
__global__ void __launch_bounds__(256)
beam_transpose_batch_kernel(const PrepSim* __restrict__ sims, int nsims,
                            const long long* __restrict__ pre) {
  __shared__ float tile[32][33];
  const long long b = blockIdx.x;
  const int si = find_segment(pre, nsims, b);
  const PrepSim& sm = sims[si];
  const int PP = sm.P * sm.P;
  const int tx = ceil_div(PP, 32), ty = sm.Np / 32;
  const long long local = b - __ldg(pre + si);
  const int f = (int)(local / ((long long)tx * ty));
  const int rem = (int)(local % ((long long)tx * ty));
  beam_transpose_tile<float>(sm.bm, sm.nant, PP, sm.Np, sm.beamT, f, (rem % tx) * 32,
                             (rem / tx) * 32, tile);
}

__global__ void __launch_bounds__(256)
ucoef_batch_kernel(const PrepSim* __restrict__ sims, int nsims, const long long* __restrict__ pre,
                   long long total) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int si = find_segment(pre, nsims, e);
    const PrepSim& sm = sims[si];
    ucoef_element<float>(sm.antpos, sm.nant, sm.Np, sm.eq2tops, 0, sm.freqs, sm.F,
                         static_cast<Ucoef32*>(sm.U), (size_t)(e - __ldg(pre + si)));
  }
}

__global__ void __launch_bounds__(256)
ubound_batch_kernel(const PrepSim* __restrict__ sims, int nsims,
                    const long long* __restrict__ pre) {
  __shared__ float red[8];
  const int si = find_segment(pre, nsims, blockIdx.x);
  const PrepSim& sm = sims[si];
  const long long l = blockIdx.x - __ldg(pre + si);
  ubound_slice(static_cast<const Ucoef32*>(sm.U) + l * sm.Np, sm.Np, sm.umax + l, red);
}

// the catalogue a simulation's records are made from: the spatially sorted
// copy, or the input when it has no sources
__device__ __forceinline__ void batch_catalogue(const PrepSim& sm, const float*& crd,
                                                const float*& I) {
  crd = sm.S > 0 ? sm.crd_s : sm.crd_eq;
  I = sm.S > 0 ? sm.I_s : sm.I_sky;
}

__global__ void __launch_bounds__(kPrepBlock)
prep_count_batch_kernel(const PrepSim* __restrict__ sims, int nsims,
                        const long long* __restrict__ pre) {
  __shared__ float rot[9];
  __shared__ int warp_cnt[kPrepBlock / 32];
  const int si = find_segment(pre, nsims, blockIdx.x);
  const PrepSim& sm = sims[si];
  const int nblk = prep_blocks_of(sm.S);
  const int local = (int)(blockIdx.x - __ldg(pre + si));
  const float *crd, *I;
  batch_catalogue(sm, crd, I);
  prep_count_block<float>(crd, sm.S, sm.eq2tops, 0, nblk, sm.blk, local % nblk, local / nblk,
                          rot, warp_cnt);
}

__global__ void __launch_bounds__(kPrepBlock)
prep_write_batch_kernel(const PrepSim* __restrict__ sims, int nsims,
                        const long long* __restrict__ pre) {
  __shared__ PrepWriteSmem<float> smw;
  const int si = find_segment(pre, nsims, blockIdx.x);
  const PrepSim& sm = sims[si];
  const int nblk = prep_blocks_of(sm.S);
  const int local = (int)(blockIdx.x - __ldg(pre + si));
  const float *crd, *I;
  batch_catalogue(sm, crd, I);
  prep_write_block<float>(crd, I, sm.S, (size_t)sm.rec_stride, sm.eq2tops, 0, nblk, sm.P, sm.blk,
                          static_cast<SrcRec32*>(sm.rec), sm.counts, local % nblk, local / nblk,
                          smw);
}

__global__ void __launch_bounds__(256)
tc_relative_batch_kernel(const PrepSim* __restrict__ sims, int nsims,
                         const long long* __restrict__ pre) {
  const int si = find_segment(pre, nsims, blockIdx.x);
  const PrepSim& sm = sims[si];
  const int nb = ceil_div(sm.rec_stride, 256);
  const int local = (int)(blockIdx.x - __ldg(pre + si));
  tc_relative_span(static_cast<SrcRec32*>(sm.rec), (size_t)sm.rec_stride, sm.counts, local / nb,
                   (local % nb) * 256);
}

cudaError_t launch_prepare_batch(const PrepSim* sims, int nsims, const PrepPre& pre,
                                 const PrepTotals& tot, int* launches, cudaStream_t st) {
  int nl = 0;
  cudaError_t e;
#define HV_PB(launch)                                 \
  do {                                                \
    launch;                                           \
    if ((e = cudaGetLastError()) != cudaSuccess) return e; \
    ++nl;                                             \
  } while (0)
  if (tot.beam > 0)
    HV_PB((beam_transpose_batch_kernel<<<(unsigned)tot.beam, dim3(32, 8), 0, st>>>(sims, nsims,
                                                                                    pre.beam)));
  if (tot.ucoef > 0)
    HV_PB((ucoef_batch_kernel<<<(unsigned)std::min<long long>((tot.ucoef + 255) / 256, 152 * 32),
                                 256, 0, st>>>(sims, nsims, pre.ucoef, tot.ucoef)));
  if (tot.slice > 0)
    HV_PB((ubound_batch_kernel<<<(unsigned)tot.slice, 256, 0, st>>>(sims, nsims, pre.slice)));
  if (tot.key > 0) {
    int k = 0;
    if ((e = launch_sort_batch(sims, nsims, pre, tot, &k, st)) != cudaSuccess) return e;
    nl += k;
  }
  if (tot.prep > 0) {
    HV_PB((prep_count_batch_kernel<<<(unsigned)tot.prep, kPrepBlock, 0, st>>>(sims, nsims,
                                                                              pre.prep)));
    HV_PB((prep_write_batch_kernel<<<(unsigned)tot.prep, kPrepBlock, 0, st>>>(sims, nsims,
                                                                              pre.prep)));
  }
  if (tot.rel > 0)
    HV_PB((tc_relative_batch_kernel<<<(unsigned)tot.rel, 256, 0, st>>>(sims, nsims, pre.rel)));
#undef HV_PB
  if (launches) *launches = nl;
  return cudaSuccess;
}

template cudaError_t launch_beam_transpose<float>(const float*, int, int, int, int, float*, cudaStream_t);
template cudaError_t launch_beam_transpose<double>(const double*, int, int, int, int, double*, cudaStream_t);
template cudaError_t launch_ucoef<float>(const float*, int, int, const float*, int, int, const double*, int, void*, cudaStream_t);
template cudaError_t launch_ucoef<double>(const double*, int, int, const double*, int, int, const double*, int, void*, cudaStream_t);
template cudaError_t launch_prep<float>(const float*, const float*, int, const float*, int, int, int, int*, void*, int*, cudaStream_t);
template cudaError_t launch_prep_strided<float>(const float*, const float*, int, const float*, int, int, int, int*, void*, size_t, int*, cudaStream_t);
template cudaError_t launch_prep<double>(const double*, const double*, int, const double*, int, int, int, int*, void*, int*, cudaStream_t);

}  // namespace hv
