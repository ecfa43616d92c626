// hv_omnical.cu -- hera_gpu's omnical redundant-calibration solver.
//
// Each problem ("pixel") p solves data[p, b] ~ g[i_b] conj(g[j_b]) u[k_b] for
// the gains g (nants) and unique baselines u (nubls) by the Omnical
// iteration of hera_gpu/redcal.py:358-743:
//   dwgts_b = |dmdl_b|^2 w_b and the weights gwgt / uwgt (their sums over
//   the baselines of each antenna / unique baseline) every check_every
//   iterations (redcal.py:590-604, kernels :117-132, :171-196);
//   gbuf / ubuf = sums of d_b = data_b conj(dmdl_b) dwgts_b / |dmdl_b|^2
//   (conjugated where the antenna is j_b; :199-236);
//   x *= (1 - gain) + gain buf / wgt (:239-280, the gain a float32 and
//   1 - gain formed in float32, redcal.py:625,630);
//   every check_every iterations (from check_after on, and at maxiter) the
//   stepped solution is checked: conv = sqrt(sum |new - old|^2 / sum |new|^2)
//   below conv_crit, or a chi^2 above the last, ends the problem keeping the
//   old solution; otherwise chisq and iters are updated (:283-354, host
//   :644-702).
//
// The reference launches a dozen kernels per iteration over 64 problems at
// a time and scatters with global atomics.  Here one launch solves every
// problem: one CTA per problem (a persistent grid that takes problems from
// a counter), every iteration inside the kernel, the solution and the
// per-baseline values in shared memory (a panel of baselines at a time when
// they do not all fit), the model recomputed from the solution where it is
// needed.  The sums over each antenna's and each unique baseline's
// baselines are gathers over a fixed incidence list (CSR), each segment
// summed by a fixed group of lanes in a fixed order, so the result does not
// depend on scheduling and repeats bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "heravis.h"
#include "hv_kernels.h"

namespace {

template <typename R> struct Cx;
template <> struct Cx<float> { using T = float2; };
template <> struct Cx<double> { using T = double2; };

// Launch and loop shape, as measured best on GB300 (float32 / float64):
//   OM_UNROLL_*  baselines a thread takes per pass of the per-baseline loops
//   OM_GATHER_*  incidence entries a lane loads ahead in the segment gathers
//   OM_MINB      CTAs of 512 threads an SM (2: 64 registers a thread)
//   OM_GK_D      float64 gathers: at least this many entries a lane
//   OM_WANT_*    CTAs of 512 threads an SM the panels of baselines are sized for
#ifndef OM_UNROLL_F
#define OM_UNROLL_F 1
#define OM_UNROLL_D 1
#define OM_GATHER_F 4
#define OM_GATHER_D 2
#endif
#ifndef OM_MINB
#define OM_MINB 2
#endif
#ifndef OM_GK_D
#define OM_GK_D 16
#endif
#ifndef OM_WANT_F
#define OM_WANT_F 2
#define OM_WANT_D 2
#endif
constexpr int kOmMaxThreads = 512;
constexpr int kOmSmemLimit = 226 * 1024;  // dynamic shared memory, below the 227 KB per CTA
constexpr int kOmThreadsPerSm = 1024 * (OM_MINB > 2 ? 2 : OM_MINB) / 2;  // register limit

template <typename R>
struct OmParams {
  int ndata, nants, nubls, nbls;
  int panel, npanels;     // baselines per panel (the last may be shorter), panels
  const uint2* bl;        // [nbls] (i | j << 16, k)
  const int* seg_off;     // [npanels][nants + nubls + 1] into seg_ent
  const uint32_t* seg_ent;// baseline within its panel | (conjugate << 31)
  const typename Cx<R>::T* data;  // [ndata][nbls]
  const R* wgts;                  // [ndata][nbls]
  typename Cx<R>::T* gains;       // [ndata][nants], in/out
  typename Cx<R>::T* ubls;        // [ndata][nubls], in/out
  R* chisq;
  R* conv;
  uint32_t* iters;
  R conv_crit;
  float gstep;
  int maxiter, check_every, check_after;
  int group;       // lanes per segment in the gathers (1, 2, 4, 8, 16 or 32)
  int* counter;    // next problem
};

template <typename C>
__device__ __forceinline__ C cmul(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
template <typename C>
__device__ __forceinline__ C conjc(C a) {
  a.y = -a.y;
  return a;
}
template <typename C>
__device__ __forceinline__ auto mag2(C a) -> decltype(a.x) {
  return a.x * a.x + a.y * a.y;
}

// g[i] conj(g[j]) u[k] (gen_dmdl, redcal.py:70-94); sol = g | u
template <typename C>
__device__ __forceinline__ C model(const C* sol, int nants, uint2 e) {
  return cmul(cmul(sol[e.x & 0xffffu], conjc(sol[e.x >> 16])), sol[nants + e.y]);
}

// Sum of three values over the block, in a fixed order; every thread gets
// the sums.  red: 3 * 32 values of shared memory.
template <typename R>
__device__ void block_sum3(R& a, R& b, R& c, R* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  __syncthreads();  // red may still be read from the last call
  if (lane == 0) {
    red[warp] = a;
    red[32 + warp] = b;
    red[64 + warp] = c;
  }
  __syncthreads();
  a = red[0];
  b = red[32];
  c = red[64];
  for (int w = 1; w < nw; ++w) {
    a += red[w];
    b += red[32 + w];
    c += red[64 + w];
  }
}

// For every segment s of the incidence list: a group of G lanes sums
// val(entry) over the segment's entries (lane l takes entries l, l + G, ...,
// kGU at a time, added in that order; then a butterfly over the group) and
// lane 0 of the group calls out(s, sum).  The loop over segments is uniform
// across the block, so every lane takes part in every shuffle.
template <int kGU, typename V, typename Val, typename Out>
__device__ __forceinline__ void seg_gather(const int* __restrict__ off,
                                           const uint32_t* __restrict__ ent, int nseg, int G,
                                           Val val, Out out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int per_warp = 32 / G, ngroups = (blockDim.x >> 5) * per_warp;
  const int gid = warp * per_warp + lane / G, gl = lane & (G - 1);
  for (int base = 0; base < nseg; base += ngroups) {
    const int s = base + gid;
    V acc = V{};
    if (s < nseg) {
      const int e1 = __ldg(off + s + 1);
      int e = __ldg(off + s) + gl;
      for (; e + (kGU - 1) * G < e1; e += kGU * G) {
        uint32_t x[kGU];
#pragma unroll
        for (int q = 0; q < kGU; ++q) x[q] = __ldg(ent + e + q * G);
#pragma unroll
        for (int q = 0; q < kGU; ++q) acc = acc + val(x[q]);
      }
      for (; e < e1; e += G) acc = acc + val(__ldg(ent + e));
    }
    for (int o = G >> 1; o > 0; o >>= 1) acc = acc + V::shfl_xor(acc, o);
    if (gl == 0 && s < nseg) out(s, acc);
  }
}

// Values summed by seg_gather.
template <typename R>
struct RealV {
  R v;
  __device__ RealV operator+(RealV o) const { return RealV{v + o.v}; }
  __device__ static RealV shfl_xor(RealV a, int o) {
    return RealV{__shfl_xor_sync(0xffffffffu, a.v, o)};
  }
};
template <typename R>
struct CplxV {
  R x, y;
  __device__ CplxV operator+(CplxV o) const { return CplxV{x + o.x, y + o.y}; }
  __device__ static CplxV shfl_xor(CplxV a, int o) {
    return CplxV{__shfl_xor_sync(0xffffffffu, a.x, o), __shfl_xor_sync(0xffffffffu, a.y, o)};
  }
};

// Baselines per thread per pass of the per-baseline loops, their loads
// issued before any of their stores.
template <typename R> struct Unroll {
  static constexpr int n = sizeof(R) == 4 ? OM_UNROLL_F : OM_UNROLL_D;
  static constexpr int gather = sizeof(R) == 4 ? OM_GATHER_F : OM_GATHER_D;  // seg_gather
};

// sum_b |data_b - model_b|^2 w_b over this thread's baselines (calc_chisq,
// redcal.py:97-114)
template <typename R, typename C>
__device__ __forceinline__ R chisq_part(const C* sol, int nants, const uint2* __restrict__ bl,
                                        const C* data, const R* wgt, int nbls) {
  constexpr int U = Unroll<R>::n;
  R acc = 0;
  for (int b0 = threadIdx.x; b0 < nbls; b0 += U * blockDim.x) {
    uint2 e[U];
    C x[U];
    R w[U];
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const int b = b0 + q * blockDim.x;
      if (b < nbls) {
        e[q] = bl[b];
        x[q] = data[b];
        w[q] = wgt[b];
      }
    }
#pragma unroll
    for (int q = 0; q < U; ++q) {
      if (b0 + q * blockDim.x < nbls) {
        const C m = model(sol, nants, e[q]);
        const R dx = x[q].x - m.x, dy = x[q].y - m.y;
        acc += (dx * dx + dy * dy) * w[q];
      }
    }
  }
  return acc;
}

// One CTA per problem.  Shared memory, per segment (antennas, then unique
// baselines): the solution and the stepped solution (complex, swapped after
// each accepted step; the stepped one also holds the partial sums of the
// panels before the last), the weights gwgt | uwgt, the magnitudes when they
// were formed and their ratios to the current ones; reduction scratch; d for
// one panel of baselines (complex; also the weights dwgts while they are
// formed); with one panel, data and w too (kDataShared), else they are read
// from global memory (the L2 keeps a problem's rows across its iterations).
//
// The baselines are taken a panel at a time: the per-baseline values of a
// panel, then its gathers, the panel sums added in panel order.  Panels keep
// the shared memory of a CTA small enough for two CTAs an SM.
//
// dwgts_b / |dmdl_b|^2 of calc_gu_buf (redcal.py:219) is
// w_b |m0_b|^2 / |m_b|^2 with m0 the model when the weights were formed;
// |m_b|^2 = |g_i|^2 |g_j|^2 |u_k|^2, so the factor is taken as
// w_b ra_i ra_j ru_k with ra = |g0|^2 / |g|^2 per antenna and ru per unique
// baseline: nants + nubls divisions an iteration instead of nbls.
template <typename R, bool kDataShared>
__global__ void __launch_bounds__(kOmMaxThreads, OM_MINB) omnical_kernel(const OmParams<R> p) {
  using C = typename Cx<R>::T;
  constexpr int U = Unroll<R>::n;
  extern __shared__ __align__(16) unsigned char smem[];
  const int nants = p.nants, nubls = p.nubls, nbls = p.nbls, nseg = nants + nubls;
  const int PB = p.panel, np = p.npanels;
  C* const solA = reinterpret_cast<C*>(smem);
  C* const solB = solA + nseg;
  R* const gw = reinterpret_cast<R*>(solB + nseg);  // gwgt | uwgt
  R* const mg0 = gw + nseg;                         // |g0|^2 | |u0|^2
  R* const ra = mg0 + nseg;                         // ratios
  R* const red = ra + nseg;                         // 96 values
  unsigned char* next = reinterpret_cast<unsigned char*>(red + 96);
  next = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(next) + 15) & ~uintptr_t(15));
  C* const d = reinterpret_cast<C*>(next);
  R* const dw = reinterpret_cast<R*>(d);
  C* const sdata = d + PB;
  R* const sw = reinterpret_cast<R*>(sdata + nbls);
  __shared__ int s_prob;

  const int tid = threadIdx.x, nt = blockDim.x;
  const R one_m = (R)(1.0f - p.gstep);  // formed in float, as the reference
  const R gs = (R)p.gstep;
  const uint2* __restrict__ bl = p.bl;

  for (;;) {
    __syncthreads();  // the last problem's reads of s_prob and shared arrays are done
    if (tid == 0) s_prob = atomicAdd(p.counter, 1);
    __syncthreads();
    const int prob = s_prob;
    if (prob >= p.ndata) return;
    const C* const gdata = p.data + (size_t)prob * nbls;
    const R* const gwgt = p.wgts + (size_t)prob * nbls;
    for (int a = tid; a < nants; a += nt) solA[a] = p.gains[(size_t)prob * nants + a];
    for (int k = tid; k < nubls; k += nt) solA[nants + k] = p.ubls[(size_t)prob * nubls + k];
    if (kDataShared) {
      for (int b = tid; b < nbls; b += nt) {
        sdata[b] = __ldg(gdata + b);
        sw[b] = __ldg(gwgt + b);
      }
    }
    const C* const data = kDataShared ? sdata : gdata;
    const R* const wgt = kDataShared ? sw : gwgt;
    __syncthreads();
    C *sol = solA, *nsol = solB;

    // chi^2 of the starting solution (redcal.py:566-577)
    R chisq = chisq_part(sol, nants, bl, data, wgt, nbls), z1 = 0, z2 = 0;
    block_sum3(chisq, z1, z2, red);
    R conv = 0;
    uint32_t iters = 0;

    for (int it = 1; it <= p.maxiter; ++it) {
      if (it % p.check_every == 1) {
        // weights from the current model (calc_dwgts, calc_gu_wgt)
        for (int s = tid; s < nseg; s += nt) {
          mg0[s] = mag2(sol[s]);
          ra[s] = 1;
        }
        for (int pn = 0; pn < np; ++pn) {
          const int b0 = pn * PB, nb = min(PB, nbls - b0);
          for (int b = tid; b < nb; b += nt) dw[b] = mag2(model(sol, nants, bl[b0 + b])) * wgt[b0 + b];
          __syncthreads();
          seg_gather<Unroll<R>::gather, RealV<R>>(
              p.seg_off + (size_t)pn * (nseg + 1), p.seg_ent, nseg, p.group,
              [&](uint32_t e) { return RealV<R>{dw[e & 0x7fffffffu]}; },
              [&](int s, RealV<R> v) { gw[s] = pn ? gw[s] + v.v : v.v; });
          __syncthreads();  // dw is overwritten below
        }
      } else {
        for (int s = tid; s < nseg; s += nt) ra[s] = mg0[s] / mag2(sol[s]);
        __syncthreads();
      }
      // d_b = data_b conj(m_b) dwgts_b / |m_b|^2 (calc_gu_buf), summed per
      // antenna and unique baseline, then the step (update_gains/_ubls)
      for (int pn = 0; pn < np; ++pn) {
        const int b0 = pn * PB, nb = min(PB, nbls - b0);
        for (int c0 = tid; c0 < nb; c0 += U * nt) {
          uint2 e[U];
          C x[U];
          R w[U];
#pragma unroll
          for (int q = 0; q < U; ++q)
            if (c0 + q * nt < nb) {
              e[q] = bl[b0 + c0 + q * nt];
              x[q] = data[b0 + c0 + q * nt];
              w[q] = wgt[b0 + c0 + q * nt];
            }
#pragma unroll
          for (int q = 0; q < U; ++q)
            if (c0 + q * nt < nb) {
              const int i = e[q].x & 0xffffu, j = e[q].x >> 16;
              const C m = model(sol, nants, e[q]);
              const R t = w[q] * ra[i] * ra[j] * ra[nants + e[q].y];
              C z = cmul(x[q], conjc(m));
              z.x *= t;
              z.y *= t;
              d[c0 + q * nt] = z;
            }
        }
        __syncthreads();
        const bool last = pn == np - 1;
        seg_gather<Unroll<R>::gather, CplxV<R>>(
            p.seg_off + (size_t)pn * (nseg + 1), p.seg_ent, nseg, p.group,
            [&](uint32_t e) {
              const C z = d[e & 0x7fffffffu];
              return CplxV<R>{z.x, (e >> 31) ? -z.y : z.y};
            },
            [&](int s, CplxV<R> v) {
              if (pn) {
                v.x = nsol[s].x + v.x;
                v.y = nsol[s].y + v.y;
              }
              C f;
              if (!last) {
                f.x = v.x;
                f.y = v.y;
                nsol[s] = f;  // partial sum
                return;
              }
              f.x = one_m + gs * v.x / gw[s];
              f.y = gs * v.y / gw[s];
              nsol[s] = cmul(sol[s], f);
            });
        __syncthreads();
      }
      const bool check = !(it < p.maxiter && (it < p.check_after || it % p.check_every != 0));
      if (!check) {
        C* t = sol; sol = nsol; nsol = t;
        continue;
      }
      // convergence and chi^2 of the stepped solution (calc_conv,
      // calc_chisq, update_active)
      R nchisq = chisq_part(nsol, nants, bl, data, wgt, nbls), csum = 0, cwgt = 0;
      for (int s = tid; s < nseg; s += nt) {
        const C x = nsol[s], y = sol[s];
        const R dx = x.x - y.x, dy = x.y - y.y;
        csum += dx * dx + dy * dy;
        cwgt += mag2(x);
      }
      block_sum3(nchisq, csum, cwgt, red);
      conv = sqrt(csum / cwgt);
      if (conv < p.conv_crit || nchisq > chisq) break;
      chisq = nchisq;
      iters = (uint32_t)it;
      C* t = sol; sol = nsol; nsol = t;
    }
    __syncthreads();
    for (int a = tid; a < nants; a += nt) p.gains[(size_t)prob * nants + a] = sol[a];
    for (int k = tid; k < nubls; k += nt) p.ubls[(size_t)prob * nubls + k] = sol[nants + k];
    if (tid == 0) {
      p.chisq[prob] = chisq;
      p.conv[prob] = conv;
      p.iters[prob] = iters;
    }
  }
}

struct Plan {
  int threads = 64, group = 1, blocks_per_sm = 1, panel = 0, npanels = 1;
  bool data_shared = false;
  size_t smem = 0;
};

// Launch shape: threads = about half the baselines (64 .. 512); everything
// in shared memory when that leaves 16 warps an SM, else panels of
// baselines sized for two CTAs (or the thread limit) an SM.
template <typename R>
int make_plan(int nants, int nubls, int nbls, Plan* out) {
  using C = typename Cx<R>::T;
  Plan pl;
  const int t = ((nbls / 2 + 31) / 32) * 32;
  pl.threads = std::max(64, std::min(kOmMaxThreads, t));
  const size_t nseg = (size_t)nants + nubls;
  const size_t fixed = (2 * sizeof(C) + 3 * sizeof(R)) * nseg + 96 * sizeof(R) + 16;
  auto per_sm = [&](size_t s) {
    return std::min(32, std::min(kOmThreadsPerSm / pl.threads, (int)((228 * 1024) / (s + 1024))));
  };
  const size_t all = fixed + (2 * sizeof(C) + sizeof(R)) * (size_t)nbls;
  if (all <= (size_t)kOmSmemLimit && per_sm(all) * pl.threads >= 512) {
    pl.data_shared = true;
    pl.panel = std::max(nbls, 1);
    pl.npanels = 1;
    pl.smem = all;
  } else {
    const int want = std::max(1, (sizeof(R) == 4 ? OM_WANT_F : OM_WANT_D) * 512 / pl.threads);
    const size_t target = std::min((size_t)kOmSmemLimit, (size_t)(228 * 1024) / want - 1024);
    if (fixed + 32 * sizeof(C) > target) return HV_ERR_ARG;
    const size_t pb = std::min((size_t)std::max(nbls, 1), (target - fixed) / sizeof(C));
    pl.npanels = (int)((nbls + pb - 1) / pb);
    pl.npanels = std::max(pl.npanels, 1);
    pl.panel = (nbls + pl.npanels - 1) / pl.npanels;
    pl.smem = fixed + sizeof(C) * (size_t)pl.panel;
  }
  pl.blocks_per_sm = std::max(1, per_sm(pl.smem));
  // lanes per segment, a power of two <= 32, from the mean segment length
  // of a panel: float32 (latency-bound) about its square root; float64
  // (bound by the FP64 pipe, where each level of the butterfly over the
  // lanes costs adds) at least OM_GK_D entries a lane
  const double mean = nseg ? 3.0 * pl.panel / nseg : 1.0;
  int g = 1;
  if (sizeof(R) == 4)
    while (g < 32 && 4.0 * g * g <= mean) g *= 2;
  else
    while (g < 32 && 2.0 * g * OM_GK_D <= mean) g *= 2;
  pl.group = g;
  *out = pl;
  return HV_OK;
}

int fail(hv_context* ctx, int code, const char* msg) {
  if (ctx) hv_context_set_error(ctx, msg);
  return code;
}

int check_indices(hv_context* ctx, const uint32_t* ggu, int nbls, int nants, int nubls) {
  char msg[200];
  for (int b = 0; b < nbls; ++b) {
    const uint32_t i = ggu[3 * b], j = ggu[3 * b + 1], k = ggu[3 * b + 2];
    if (i >= (uint32_t)nants || j >= (uint32_t)nants || k >= (uint32_t)nubls) {
      snprintf(msg, sizeof msg, "omnical: baseline %d indexes (%u, %u, %u) out of range "
               "(%d antennas, %d unique baselines)", b, i, j, k, nants, nubls);
      return fail(ctx, HV_ERR_ARG, msg);
    }
  }
  return HV_OK;
}

// Incidence lists of the baselines, one per panel of `panel` baselines: for
// antenna a, the panel's baselines with i == a (as is) and j == a
// (conjugated); for unique baseline k, those with k; entries hold the
// baseline's index within its panel.
void build_csr(const uint32_t* ggu, int nbls, int nants, int nubls, int panel, int npanels,
               std::vector<uint2>& bl, std::vector<int>& off, std::vector<uint32_t>& ent) {
  const int nseg = nants + nubls;
  bl.resize(nbls);
  off.assign((size_t)npanels * (nseg + 1), 0);
  ent.resize((size_t)3 * nbls);
  size_t base = 0;
  for (int pn = 0; pn < npanels; ++pn) {
    const int b0 = pn * panel, b1 = std::min(nbls, b0 + panel);
    int* o = off.data() + (size_t)pn * (nseg + 1);
    std::vector<int> cnt(nseg + 1, 0);
    for (int b = b0; b < b1; ++b) {
      cnt[ggu[3 * b] + 1]++;
      cnt[ggu[3 * b + 1] + 1]++;
      cnt[nants + ggu[3 * b + 2] + 1]++;
    }
    o[0] = (int)base;
    for (int s = 0; s < nseg; ++s) o[s + 1] = o[s] + cnt[s + 1];
    std::vector<int> pos(o, o + nseg);
    for (int b = b0; b < b1; ++b) {
      const uint32_t i = ggu[3 * b], j = ggu[3 * b + 1], k = ggu[3 * b + 2];
      bl[b] = make_uint2(i | (j << 16), k);
      ent[pos[i]++] = (uint32_t)(b - b0);
      ent[pos[j]++] = (uint32_t)(b - b0) | 0x80000000u;
      ent[pos[nants + k]++] = (uint32_t)(b - b0);
    }
    base = (size_t)o[nseg];
  }
}

int check_sizes(hv_context* ctx, int precision, int nbls, int nants, int nubls, int ndata,
                int maxiter, int check_every) {
  char msg[200];
  if ((precision != 1 && precision != 2) || nbls < 0 || nants < 0 || nubls < 0 || ndata < 0 ||
      maxiter < 0 || check_every <= 1 || nants > 65535 || nbls > 0x7fffffff / 3) {
    snprintf(msg, sizeof msg, "omnical: bad arguments (precision %d, %d baselines, %d antennas, "
             "%d unique baselines, %d problems, maxiter %d, check_every %d)", precision, nbls,
             nants, nubls, ndata, maxiter, check_every);
    return fail(ctx, HV_ERR_ARG, msg);
  }
  return HV_OK;
}

template <typename R>
int run_typed(hv_context* ctx, const uint32_t* ggu, int nbls, void* d_gains, int nants,
              void* d_ubls, int nubls, const void* d_data, const void* d_wgts, int ndata,
              double conv_crit, int maxiter, int check_every, int check_after, double gain,
              void* d_chisq, uint32_t* d_iters, void* d_conv, cudaStream_t st) {
  int r = check_indices(ctx, ggu, nbls, nants, nubls);
  if (r != HV_OK) return r;
  if (ndata == 0) return HV_OK;
  Plan pl;
  if (make_plan<R>(nants, nubls, nbls, &pl) != HV_OK)
    return fail(ctx, HV_ERR_ARG, "omnical: too many antennas and unique baselines for one CTA");
  std::vector<uint2> bl;
  std::vector<int> off;
  std::vector<uint32_t> ent;
  build_csr(ggu, nbls, nants, nubls, pl.panel, pl.npanels, bl, off, ent);
  const int nsm = std::max(1, hv_context_num_sms(ctx));
  const int grid = std::max(1, std::min(ndata, pl.blocks_per_sm * nsm));
  const size_t n_bl = sizeof(uint2) * bl.size(), n_off = sizeof(int) * off.size(),
               n_ent = sizeof(uint32_t) * ent.size();
  const size_t o_off = (n_bl + 255) & ~size_t(255);
  const size_t o_ent = (o_off + n_off + 255) & ~size_t(255);
  const size_t o_cnt = (o_ent + n_ent + 255) & ~size_t(255);
  const size_t total = o_cnt + 256;
  void* buf = nullptr;
  if (cudaMallocAsync(&buf, total, st) != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, HV_ERR_OOM, "omnical: device allocation failed");
  }
  char* b8 = static_cast<char*>(buf);
  r = HV_OK;
  if ((n_bl && cudaMemcpyAsync(b8, bl.data(), n_bl, cudaMemcpyHostToDevice, st) != cudaSuccess) ||
      cudaMemcpyAsync(b8 + o_off, off.data(), n_off, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      (n_ent && cudaMemcpyAsync(b8 + o_ent, ent.data(), n_ent, cudaMemcpyHostToDevice, st) !=
                    cudaSuccess) ||
      cudaMemsetAsync(b8 + o_cnt, 0, sizeof(int), st) != cudaSuccess)
    r = HV_ERR_CUDA;
  if (r == HV_OK) {
    static bool configured[2] = {false, false};
    if (!configured[sizeof(R) == 8]) {
      for (const void* k : {reinterpret_cast<const void*>(omnical_kernel<R, false>),
                            reinterpret_cast<const void*>(omnical_kernel<R, true>)})
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kOmSmemLimit) !=
            cudaSuccess)
          r = HV_ERR_CUDA;
      if (r == HV_OK) configured[sizeof(R) == 8] = true;
    }
  }
  if (r == HV_OK) {
    using C = typename Cx<R>::T;
    OmParams<R> p;
    p.ndata = ndata;
    p.nants = nants;
    p.nubls = nubls;
    p.nbls = nbls;
    p.panel = pl.panel;
    p.npanels = pl.npanels;
    p.bl = reinterpret_cast<const uint2*>(b8);
    p.seg_off = reinterpret_cast<const int*>(b8 + o_off);
    p.seg_ent = reinterpret_cast<const uint32_t*>(b8 + o_ent);
    p.data = static_cast<const C*>(d_data);
    p.wgts = static_cast<const R*>(d_wgts);
    p.gains = static_cast<C*>(d_gains);
    p.ubls = static_cast<C*>(d_ubls);
    p.chisq = static_cast<R*>(d_chisq);
    p.conv = static_cast<R*>(d_conv);
    p.iters = d_iters;
    p.conv_crit = (R)conv_crit;
    p.gstep = (float)gain;
    p.maxiter = maxiter;
    p.check_every = check_every;
    p.check_after = check_after;
    p.group = pl.group;
    p.counter = reinterpret_cast<int*>(b8 + o_cnt);
    if (pl.data_shared)
      omnical_kernel<R, true><<<grid, pl.threads, pl.smem, st>>>(p);
    else
      omnical_kernel<R, false><<<grid, pl.threads, pl.smem, st>>>(p);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      hv_context_set_error(ctx, cudaGetErrorString(e));
      r = HV_ERR_CUDA;
    } else {
      hv_context_add_launches(ctx, 1);
    }
  }
  cudaFreeAsync(buf, st);
  return r;
}

int run_device(hv_context* ctx, int precision, const uint32_t* ggu, int nbls, void* d_gains,
               int nants, void* d_ubls, int nubls, const void* d_data, const void* d_wgts,
               int ndata, double conv_crit, int maxiter, int check_every, int check_after,
               double gain, void* d_chisq, uint32_t* d_iters, void* d_conv, cudaStream_t st) {
  if (precision == 1)
    return run_typed<float>(ctx, ggu, nbls, d_gains, nants, d_ubls, nubls, d_data, d_wgts,
                            ndata, conv_crit, maxiter, check_every, check_after, gain, d_chisq,
                            d_iters, d_conv, st);
  return run_typed<double>(ctx, ggu, nbls, d_gains, nants, d_ubls, nubls, d_data, d_wgts, ndata,
                           conv_crit, maxiter, check_every, check_after, gain, d_chisq, d_iters,
                           d_conv, st);
}

}  // namespace

extern "C" {

int hv_omnical_device(hv_context* ctx, int precision, const uint32_t* ggu, int nbls,
                      void* d_gains, int nants, void* d_ubls, int nubls, const void* d_data,
                      const void* d_wgts, int ndata, double conv_crit, int maxiter,
                      int check_every, int check_after, double gain, void* d_chisq,
                      uint32_t* d_iters, void* d_conv, void* stream) {
  if (!ctx) return HV_ERR_ARG;
  int r = check_sizes(ctx, precision, nbls, nants, nubls, ndata, maxiter, check_every);
  if (r != HV_OK) return r;
  if (ndata > 0 && (!d_gains || !d_chisq || !d_iters || !d_conv || (nbls > 0 && (!ggu || !d_data || !d_wgts)) ||
                    (nubls > 0 && !d_ubls)))
    return fail(ctx, HV_ERR_ARG, "omnical: null buffer");
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : hv_context_stream(ctx);
  return run_device(ctx, precision, ggu, nbls, d_gains, nants, d_ubls, nubls, d_data, d_wgts,
                    ndata, conv_crit, maxiter, check_every, check_after, gain, d_chisq, d_iters,
                    d_conv, st);
}

int hv_omnical(hv_context* ctx, int precision, const uint32_t* ggu, int nbls, void* gains,
               int nants, void* ubls, int nubls, const void* data, const void* wgts, int ndata,
               double conv_crit, int maxiter, int check_every, int check_after, double gain,
               void* chisq, uint32_t* iters, void* conv) {
  if (!ctx) return HV_ERR_ARG;
  int r = check_sizes(ctx, precision, nbls, nants, nubls, ndata, maxiter, check_every);
  if (r != HV_OK) return r;
  if (ndata == 0) return (nbls > 0 && !ggu) ? HV_ERR_ARG : check_indices(ctx, ggu, nbls, nants, nubls);
  if (!gains || !chisq || !iters || !conv || (nbls > 0 && (!ggu || !data || !wgts)) ||
      (nubls > 0 && !ubls))
    return fail(ctx, HV_ERR_ARG, "omnical: null buffer");
  const size_t rs = precision == 1 ? 4 : 8;
  const size_t n_g = 2 * rs * (size_t)ndata * nants, n_u = 2 * rs * (size_t)ndata * nubls;
  const size_t n_d = 2 * rs * (size_t)ndata * nbls, n_w = rs * (size_t)ndata * nbls;
  const size_t n_c = rs * (size_t)ndata, n_i = sizeof(uint32_t) * (size_t)ndata;
  size_t o[7], tot = 0;
  const size_t sz[7] = {n_g, n_u, n_d, n_w, n_c, n_c, n_i};
  for (int i = 0; i < 7; ++i) {
    o[i] = tot;
    tot += (sz[i] + 255) & ~size_t(255);
  }
  cudaStream_t st = hv_context_stream(ctx);
  void* buf = nullptr;
  if (cudaMallocAsync(&buf, tot, st) != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, HV_ERR_OOM, "omnical: device allocation failed");
  }
  char* b = static_cast<char*>(buf);
  r = HV_OK;
  const void* src[4] = {gains, ubls, data, wgts};
  for (int i = 0; i < 4 && r == HV_OK; ++i)
    if (sz[i] && cudaMemcpyAsync(b + o[i], src[i], sz[i], cudaMemcpyHostToDevice, st) !=
                     cudaSuccess)
      r = HV_ERR_CUDA;
  if (r == HV_OK)
    r = run_device(ctx, precision, ggu, nbls, b + o[0], nants, b + o[1], nubls, b + o[2],
                   b + o[3], ndata, conv_crit, maxiter, check_every, check_after, gain, b + o[4],
                   reinterpret_cast<uint32_t*>(b + o[6]), b + o[5], st);
  void* dst[7] = {gains, ubls, nullptr, nullptr, chisq, conv, iters};
  for (int i : {0, 1, 4, 5, 6})
    if (r == HV_OK && sz[i] &&
        cudaMemcpyAsync(dst[i], b + o[i], sz[i], cudaMemcpyDeviceToHost, st) != cudaSuccess)
      r = HV_ERR_CUDA;
  cudaFreeAsync(buf, st);
  const cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess && r == HV_OK) {
    hv_context_set_error(ctx, cudaGetErrorString(e));
    r = HV_ERR_CUDA;
  }
  return r;
}

}  // extern "C"
