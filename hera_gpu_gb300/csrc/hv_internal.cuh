// hv_internal.cuh -- device-side data layouts and helpers shared by the
// kernels of libheravis.so.
//
// Data layout in HBM (one call):
//   beamT   [nfreq][P*P][Np]      beam transposed so the antennas of one beam
//                                 pixel are contiguous (coalesced gathers when
//                                 the lanes of a warp are antennas)
//   ucoef   [ntimes][nfreq][Np]   per (time, frequency, antenna) phase
//                                 coefficients U = nu/c * eq2top^T p, so that
//                                 the phase in cycles is U . s_eq
//   srcrec  [nsrc]                per time: the sources above the horizon, in
//                                 input order, one record each (below)
//   partial [nchunk][2][Np][Np]   split-K partial sums over source chunks,
//                                 plane 0 = Re V, plane 1 = Im V, stored
//                                 [b][a] (a = row antenna, b = column antenna)
// Np is nant rounded up to a multiple of 128; padded antennas have a zero
// beam and so a zero phasor.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace hv {

constexpr double kSpeedOfLight = 299792458.0;  // m/s (hera_gpu/vis.py:4,8)
constexpr int kAntPad = 128;                   // Np granularity
constexpr int kPrepBlock = 1024;               // threads per prep block

// One source above the horizon at one time (precision 1): the equatorial
// direction (for the phase), sqrt(I), and the bilinear beam corner + weights.
struct alignas(32) SrcRec32 {
  float sx, sy, sz, amp;
  int pix;      // index (py * P + px) of the lower corner in the beam
  float fx, fy; // fractional position inside the beam pixel, in [0, 1]
  int pad;
};

// precision 2
struct alignas(16) SrcRec64 {
  double sx, sy, sz, amp, fx, fy;
  int pix;
  int pad[3];
};

// Phase coefficients of one antenna at one (time, frequency).  Precision 1
// keeps U as an unevaluated float pair U = hi + lo (about 48 significant
// bits) so that the phase can be reduced to cycles exactly in FP32 (see
// phase_cycles32); precision 2 keeps plain doubles.
struct alignas(16) Ucoef32 {
  float hx, hy, hz, p0;
  float lx, ly, lz, p1;
};
struct alignas(32) Ucoef64 {
  double x, y, z, p;
};

template <typename R> struct Traits;
template <> struct Traits<float> {
  using Rec = SrcRec32;
  using U = Ucoef32;
  using C = float2;
};
template <> struct Traits<double> {
  using Rec = SrcRec64;
  using U = Ucoef64;
  using C = double2;
};

// v0 (1 - t) + v1 t written as two FMAs (hera_gpu/vis.py:29-32).
__device__ __forceinline__ float lerp(float v0, float v1, float t) {
  return fmaf(t, v1, fmaf(-t, v0, v0));
}
__device__ __forceinline__ double lerp(double v0, double v1, double t) {
  return fma(t, v1, fma(-t, v0, v0));
}

// Phase of antenna coefficients u at direction s, in cycles, reduced to
// [-0.5, 0.5].  U_k * s_k is formed as an exact float pair (product p_k plus
// its FMA residual e_k); p_k - rint(p_k) is exact for |p_k| < 2^23 (the two
// operands are within a factor of two, or the rint is 0), so the integer
// cycles are removed without rounding.  What is left -- three numbers in
// [-0.5, 0.5] plus residuals and the lo part of U -- is summed in FP32,
// giving an absolute phase error of a few 1e-8 cycles regardless of how many
// thousand cycles the baseline spans.  This replaces an FP64 product per
// (antenna, source): GB300 issues FP32 about sixty times faster than FP64.
__device__ __forceinline__ float phase_cycles32(const Ucoef32& u, float sx,
                                                float sy, float sz) {
  const float p0 = __fmul_rn(u.hx, sx);
  const float p1 = __fmul_rn(u.hy, sy);
  const float p2 = __fmul_rn(u.hz, sz);
  const float e0 = fmaf(u.hx, sx, -p0);
  const float e1 = fmaf(u.hy, sy, -p1);
  const float e2 = fmaf(u.hz, sz, -p2);
  const float r0 = __fsub_rn(p0, rintf(p0));
  const float r1 = __fsub_rn(p1, rintf(p1));
  const float r2 = __fsub_rn(p2, rintf(p2));
  const float lo = fmaf(u.lx, sx, fmaf(u.ly, sy, fmaf(u.lz, sz, __fadd_rn(__fadd_rn(e0, e1), e2))));
  const float ph = __fadd_rn(__fadd_rn(r0, r1), __fadd_rn(r2, lo));
  return __fsub_rn(ph, rintf(ph));
}

__device__ __forceinline__ double phase_cycles64(const Ucoef64& u, double sx,
                                                 double sy, double sz) {
  const double ph = fma(u.x, sx, fma(u.y, sy, u.z * sz));
  return ph - rint(ph);
}

// Bilinear beam value of antenna a for a source record (texel semantics of
// hera_gpu/vis.py:75-84; corner clamping done when the record was built).
template <typename R, typename Rec>
__device__ __forceinline__ R beam_bilinear(const R* __restrict__ beamT, int Np,
                                           int a, const Rec& r, int dx, int dy) {
  const R* b = beamT + (size_t)r.pix * Np + a;
  const R b00 = __ldg(b);
  const R b01 = __ldg(b + (size_t)dx * Np);
  const R b10 = __ldg(b + (size_t)dy * Np);
  const R b11 = __ldg(b + (size_t)(dx + dy) * Np);
  return lerp(lerp(b00, b01, (R)r.fx), lerp(b10, b11, (R)r.fx), (R)r.fy);
}

// v[a, s] for the plain path (precision 1): beam * sqrt(I) * exp(+2 pi i phi)
// with sincospi of the exactly reduced phase.
__device__ __forceinline__ float2 phasor32(const SrcRec32& r, const Ucoef32& u,
                                           float A) {
  const float ph = phase_cycles32(u, r.sx, r.sy, r.sz);
  float s, c;
  sincospif(2.0f * ph, &s, &c);
  const float amp = A * r.amp;
  return make_float2(amp * c, amp * s);
}

__device__ __forceinline__ double2 phasor64(const SrcRec64& r, const Ucoef64& u,
                                            double A) {
  const double ph = phase_cycles64(u, r.sx, r.sy, r.sz);
  double s, c;
  sincospi(2.0 * ph, &s, &c);
  const double amp = A * r.amp;
  return make_double2(amp * c, amp * s);
}

__host__ __device__ inline int ceil_div(long long a, long long b) {
  return (int)((a + b - 1) / b);
}

// Segment of flattened index x: the largest i < n with pre[i] <= x (pre:
// n + 1 non-decreasing prefix sums starting at 0).
__device__ __forceinline__ int find_segment(const long long* __restrict__ pre, int n,
                                            long long x) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(pre + mid) <= x) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

}  // namespace hv
