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
// per-baseline arrays in shared memory, the model recomputed from the
// solution where it is needed.  The sums over each antenna's and each unique
// baseline's baselines are gathers over a fixed incidence list (CSR), each
// segment summed by a fixed group of lanes in a fixed order, so the result
// does not depend on scheduling and repeats bit for bit.
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

constexpr int kOmMaxThreads = 512;
#ifndef OM_UNROLL_F
#define OM_UNROLL_F 1
#define OM_UNROLL_D 1
#define OM_GATHER_F 4
#define OM_GATHER_D 2
#endif
#ifndef OM_MINB
#define OM_MINB 2  // CTAs of 512 threads an SM: 64 registers a thread
#endif
constexpr int kOmSmemLimit = 226 * 1024;  // dynamic shared memory, below the 227 KB per CTA

// Which per-baseline arrays live in shared memory (otherwise: d in a per-CTA
// global workspace, data and wgts read from the inputs).
enum : int { kOmSmemD = 1, kOmSmemData = 2 };

template <typename R>
struct OmParams {
  int ndata, nants, nubls, nbls;
  const uint2* bl;        // [nbls] (i | j << 16, k)
  const int* seg_off;     // [nants + nubls + 1]: antennas, then unique baselines
  const uint32_t* seg_ent;// baseline | (conjugate << 31)
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
  char* ws;        // per-CTA workspace for the arrays not in shared memory
  size_t ws_stride;
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

// g[i] conj(g[j]) u[k] (gen_dmdl, redcal.py:70-94)
template <typename C>
__device__ __forceinline__ C model(const C* g, const C* u, uint2 e) {
  return cmul(cmul(g[e.x & 0xffffu], conjc(g[e.x >> 16])), u[e.y]);
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
__device__ __forceinline__ R chisq_part(const C* g, const C* u, const uint2* __restrict__ bl,
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
        const C m = model(g, u, e[q]);
        const R dx = x[q].x - m.x, dy = x[q].y - m.y;
        acc += (dx * dx + dy * dy) * w[q];
      }
    }
  }
  return acc;
}

// One CTA per problem.  Shared memory: g, gn (nants) and u, un (nubls)
// complex; gw, mg0, ra (nants) and uw, mu0, ru (nubls) real; reduction
// scratch; then d (complex, per baseline; also the weights dwgts on the
// iterations that form them) and data (complex) and w, if they fit
// (OmParams::in_smem), else d in the per-CTA workspace and data and w read
// from the inputs.
//
// dwgts_b / |dmdl_b|^2 of calc_gu_buf (redcal.py:219) is
// w_b |m0_b|^2 / |m_b|^2 with m0 the model when the weights were formed;
// |m_b|^2 = |g_i|^2 |g_j|^2 |u_k|^2, so the factor is taken as
// w_b ra_i ra_j ru_k with ra = |g0|^2 / |g|^2 per antenna and ru per unique
// baseline: nants + nubls divisions an iteration instead of nbls.
template <typename R, int kLayout>
__global__ void __launch_bounds__(kOmMaxThreads, OM_MINB) omnical_kernel(const OmParams<R> p) {
  using C = typename Cx<R>::T;
  constexpr int U = Unroll<R>::n;
  constexpr bool kDShared = (kLayout & kOmSmemD) != 0, kDataShared = (kLayout & kOmSmemData) != 0;
  extern __shared__ __align__(16) unsigned char smem[];
  const int nants = p.nants, nubls = p.nubls, nbls = p.nbls, nseg = nants + nubls;
  C* gA = reinterpret_cast<C*>(smem);
  C* gB = gA + nants;
  C* uA = gB + nants;
  C* uB = uA + nubls;
  R* gw = reinterpret_cast<R*>(uB + nubls);  // gw | uw
  R* uw = gw + nants;
  R* mg0 = uw + nubls;                        // mg0 | mu0
  R* mu0 = mg0 + nants;
  R* ra = mu0 + nubls;                        // ra | ru
  R* ru = ra + nants;
  R* red = ru + nubls;  // 96 values
  unsigned char* next = reinterpret_cast<unsigned char*>(red + 96);
  next = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(next) + 15) & ~uintptr_t(15));
  C* const d = kDShared ? reinterpret_cast<C*>(next)
                        : reinterpret_cast<C*>(p.ws + (size_t)blockIdx.x * p.ws_stride);
  R* const dw = reinterpret_cast<R*>(d);
  C* const sdata = reinterpret_cast<C*>(next + sizeof(C) * (size_t)nbls);
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
    for (int a = tid; a < nants; a += nt) gA[a] = p.gains[(size_t)prob * nants + a];
    for (int k = tid; k < nubls; k += nt) uA[k] = p.ubls[(size_t)prob * nubls + k];
    if (kDataShared) {
      for (int b = tid; b < nbls; b += nt) {
        sdata[b] = __ldg(gdata + b);
        sw[b] = __ldg(gwgt + b);
      }
    }
    const C* const data = kDataShared ? sdata : gdata;
    const R* const wgt = kDataShared ? sw : gwgt;
    __syncthreads();
    C *g = gA, *gn = gB, *u = uA, *un = uB;

    // chi^2 of the starting solution (redcal.py:566-577)
    R chisq = chisq_part(g, u, bl, data, wgt, nbls), z1 = 0, z2 = 0;
    block_sum3(chisq, z1, z2, red);
    R conv = 0;
    uint32_t iters = 0;

    for (int it = 1; it <= p.maxiter; ++it) {
      if (it % p.check_every == 1) {
        // weights from the current model (calc_dwgts, calc_gu_wgt)
        for (int s = tid; s < nseg; s += nt) {
          const C x = s < nants ? g[s] : u[s - nants];
          mg0[s] = mag2(x);
          ra[s] = 1;
        }
        for (int b0 = tid; b0 < nbls; b0 += U * nt) {
          uint2 e[U];
          R w[U];
#pragma unroll
          for (int q = 0; q < U; ++q)
            if (b0 + q * nt < nbls) {
              e[q] = bl[b0 + q * nt];
              w[q] = wgt[b0 + q * nt];
            }
#pragma unroll
          for (int q = 0; q < U; ++q)
            if (b0 + q * nt < nbls) dw[b0 + q * nt] = mag2(model(g, u, e[q])) * w[q];
        }
        __syncthreads();
        seg_gather<Unroll<R>::gather, RealV<R>>(
            p.seg_off, p.seg_ent, nseg, p.group,
            [&](uint32_t e) { return RealV<R>{dw[e & 0x7fffffffu]}; },
            [&](int s, RealV<R> v) { gw[s] = v.v; });
        __syncthreads();  // dw is overwritten by d below
      } else {
        for (int s = tid; s < nseg; s += nt) {
          const C x = s < nants ? g[s] : u[s - nants];
          ra[s] = mg0[s] / mag2(x);
        }
        __syncthreads();
      }
      // d_b = data_b conj(m_b) dwgts_b / |m_b|^2 (calc_gu_buf)
      for (int b0 = tid; b0 < nbls; b0 += U * nt) {
        uint2 e[U];
        C x[U];
        R w[U];
#pragma unroll
        for (int q = 0; q < U; ++q)
          if (b0 + q * nt < nbls) {
            e[q] = bl[b0 + q * nt];
            x[q] = data[b0 + q * nt];
            w[q] = wgt[b0 + q * nt];
          }
#pragma unroll
        for (int q = 0; q < U; ++q)
          if (b0 + q * nt < nbls) {
            const int i = e[q].x & 0xffffu, j = e[q].x >> 16;
            const C m = model(g, u, e[q]);
            const R t = w[q] * ra[i] * ra[j] * ru[e[q].y];
            C z = cmul(x[q], conjc(m));
            z.x *= t;
            z.y *= t;
            d[b0 + q * nt] = z;
          }
      }
      __syncthreads();
      // the stepped solution (update_gains / update_ubls)
      seg_gather<Unroll<R>::gather, CplxV<R>>(
          p.seg_off, p.seg_ent, nseg, p.group,
          [&](uint32_t e) {
            const C z = d[e & 0x7fffffffu];
            return CplxV<R>{z.x, (e >> 31) ? -z.y : z.y};
          },
          [&](int s, CplxV<R> v) {
            C f;
            f.x = one_m + gs * v.x / gw[s];
            f.y = gs * v.y / gw[s];
            if (s < nants) gn[s] = cmul(g[s], f);
            else un[s - nants] = cmul(u[s - nants], f);
          });
      __syncthreads();
      const bool check = !(it < p.maxiter && (it < p.check_after || it % p.check_every != 0));
      if (!check) {
        C* t = g; g = gn; gn = t;
        t = u; u = un; un = t;
        continue;
      }
      // convergence and chi^2 of the stepped solution (calc_conv,
      // calc_chisq, update_active)
      R nchisq = chisq_part(gn, un, bl, data, wgt, nbls), csum = 0, cwgt = 0;
      for (int s = tid; s < nseg; s += nt) {
        const C x = s < nants ? gn[s] : un[s - nants];
        const C y = s < nants ? g[s] : u[s - nants];
        const R dx = x.x - y.x, dy = x.y - y.y;
        csum += dx * dx + dy * dy;
        cwgt += mag2(x);
      }
      block_sum3(nchisq, csum, cwgt, red);
      conv = sqrt(csum / cwgt);
      if (conv < p.conv_crit || nchisq > chisq) break;
      chisq = nchisq;
      iters = (uint32_t)it;
      C* t = g; g = gn; gn = t;
      t = u; u = un; un = t;
    }
    __syncthreads();
    for (int a = tid; a < nants; a += nt) p.gains[(size_t)prob * nants + a] = g[a];
    for (int k = tid; k < nubls; k += nt) p.ubls[(size_t)prob * nubls + k] = u[k];
    if (tid == 0) {
      p.chisq[prob] = chisq;
      p.conv[prob] = conv;
      p.iters[prob] = iters;
    }
  }
}

struct Plan {
  int threads = 64, group = 1, in_smem = 0, blocks_per_sm = 1;
  size_t smem = 0, ws_stride = 0;
};

template <typename R>
Plan make_plan(int nants, int nubls, int nbls, int nsm_threads_cap) {
  using C = typename Cx<R>::T;
  Plan pl;
  int t = ((nbls / 2 + 31) / 32) * 32;
  pl.threads = std::max(64, std::min(kOmMaxThreads, t));
  const size_t fixed =
      (2 * sizeof(C) + 3 * sizeof(R)) * (size_t)(nants + nubls) + 96 * sizeof(R) + 16;
  const size_t pd = sizeof(C) * (size_t)nbls;
  const size_t pdata = (sizeof(C) + sizeof(R)) * (size_t)nbls;
  const int options[3] = {kOmSmemD | kOmSmemData, kOmSmemD, 0};
  auto bytes = [&](int f) {
    return fixed + ((f & kOmSmemD) ? pd : 0) + ((f & kOmSmemData) ? pdata : 0);
  };
  auto per_sm = [&](size_t s) {
    return std::min(32, std::min(nsm_threads_cap / pl.threads, (int)((228 * 1024) / (s + 1024))));
  };
  // the first layout that keeps at least 16 warps per SM, else the one
  // with the most
  int best = -1, best_threads = -1;
  for (int i = 0; i < 3; ++i) {
    const size_t s = bytes(options[i]);
    if (s > (size_t)kOmSmemLimit) continue;
    const int bps = per_sm(s);
    if (bps < 1) continue;
    if (bps * pl.threads >= 512) {
      best = i;
      break;
    }
    if (bps * pl.threads > best_threads) {
      best = i;
      best_threads = bps * pl.threads;
    }
  }
  if (best < 0) best = 2;
  pl.in_smem = options[best];
  pl.smem = bytes(pl.in_smem);
  pl.ws_stride = (pl.in_smem & kOmSmemD) ? 0 : (pd + 255) & ~size_t(255);
  pl.blocks_per_sm = std::max(1, per_sm(pl.smem));
  // lanes per segment: about the mean segment length, a power of two <= 32
  const double mean = (nants + nubls) ? 3.0 * nbls / (nants + nubls) : 1.0;
  int g = 1;
  while (g < 32 && 2 * g <= mean) g *= 2;
  pl.group = g;
  return pl;
}

int fail(hv_context* ctx, int code, const char* msg) {
  if (ctx) hv_context_set_error(ctx, msg);
  return code;
}

// Incidence lists of the baselines: for antenna a, the baselines with i == a
// (as is) and j == a (conjugated); for unique baseline k, those with k.
int build_csr(hv_context* ctx, const uint32_t* ggu, int nbls, int nants, int nubls,
              std::vector<uint2>& bl, std::vector<int>& off, std::vector<uint32_t>& ent) {
  char msg[200];
  bl.resize(nbls);
  const int nseg = nants + nubls;
  off.assign(nseg + 1, 0);
  for (int b = 0; b < nbls; ++b) {
    const uint32_t i = ggu[3 * b], j = ggu[3 * b + 1], k = ggu[3 * b + 2];
    if (i >= (uint32_t)nants || j >= (uint32_t)nants || k >= (uint32_t)nubls) {
      snprintf(msg, sizeof msg, "omnical: baseline %d indexes (%u, %u, %u) out of range "
               "(%d antennas, %d unique baselines)", b, i, j, k, nants, nubls);
      return fail(ctx, HV_ERR_ARG, msg);
    }
    bl[b] = make_uint2(i | (j << 16), k);
    off[i + 1]++;
    off[j + 1]++;
    off[nants + k + 1]++;
  }
  for (int s = 0; s < nseg; ++s) off[s + 1] += off[s];
  ent.resize((size_t)off[nseg]);
  std::vector<int> pos(off.begin(), off.end() - 1);
  for (int b = 0; b < nbls; ++b) {
    const uint32_t i = ggu[3 * b], j = ggu[3 * b + 1], k = ggu[3 * b + 2];
    ent[pos[i]++] = (uint32_t)b;
    ent[pos[j]++] = (uint32_t)b | 0x80000000u;
    ent[pos[nants + k]++] = (uint32_t)b;
  }
  return HV_OK;
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
  std::vector<uint2> bl;
  std::vector<int> off;
  std::vector<uint32_t> ent;
  int r = build_csr(ctx, ggu, nbls, nants, nubls, bl, off, ent);
  if (r != HV_OK) return r;
  if (ndata == 0) return HV_OK;
  const int nsm = std::max(1, hv_context_num_sms(ctx));
  const Plan pl = make_plan<R>(nants, nubls, nbls, 1024);  // 64 registers a thread
  if (pl.smem > (size_t)kOmSmemLimit && pl.in_smem == 0)
    return fail(ctx, HV_ERR_ARG, "omnical: too many antennas and unique baselines for one CTA");
  const int grid = std::max(1, std::min(ndata, pl.blocks_per_sm * nsm));
  const size_t n_bl = sizeof(uint2) * bl.size(), n_off = sizeof(int) * off.size(),
               n_ent = sizeof(uint32_t) * ent.size();
  const size_t o_off = (n_bl + 255) & ~size_t(255);
  const size_t o_ent = (o_off + n_off + 255) & ~size_t(255);
  const size_t o_cnt = (o_ent + n_ent + 255) & ~size_t(255);
  const size_t o_ws = o_cnt + 256;
  const size_t total = o_ws + pl.ws_stride * (size_t)grid;
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
      for (const void* k : {reinterpret_cast<const void*>(omnical_kernel<R, 0>),
                            reinterpret_cast<const void*>(omnical_kernel<R, kOmSmemD>),
                            reinterpret_cast<const void*>(omnical_kernel<R, kOmSmemD | kOmSmemData>)})
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
    p.ws = b8 + o_ws;
    p.ws_stride = pl.ws_stride;
    p.counter = reinterpret_cast<int*>(b8 + o_cnt);
    if (pl.in_smem == (kOmSmemD | kOmSmemData))
      omnical_kernel<R, kOmSmemD | kOmSmemData><<<grid, pl.threads, pl.smem, st>>>(p);
    else if (pl.in_smem == kOmSmemD)
      omnical_kernel<R, kOmSmemD><<<grid, pl.threads, pl.smem, st>>>(p);
    else
      omnical_kernel<R, 0><<<grid, pl.threads, pl.smem, st>>>(p);
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
  if (ndata == 0) {
    std::vector<uint2> bl;
    std::vector<int> off;
    std::vector<uint32_t> ent;
    return build_csr(ctx, ggu, nbls, nants, nubls, bl, off, ent);
  }
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
