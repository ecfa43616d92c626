// hv_sort.cu -- spatial ordering of the source catalogue for the fused path.
//
// The visibility sum is over sources, so their order is free.  Putting
// sources that are close on the sky next to each other makes the 32 sources
// of a pipeline stage fall on the same few beam pixels: the beam gathers of a
// stage hit L1, and the phase of a source can be taken relative to a nearby
// reference source.  Rotation to topocentric is an isometry, so an order
// that is local on the equatorial sphere stays local at every time.
//
// Key: Morton code (16 bits per axis) of the octahedral projection of the
// unit vector.  Sort: bitonic network on (key << 32 | index) -- a total
// order, so the permutation (and every result downstream) is deterministic.
#include <algorithm>

#include "hv_internal.cuh"
#include "hv_kernels.h"

namespace hv {

__device__ __forceinline__ uint32_t spread16(uint32_t a) {
  a = (a | (a << 8)) & 0x00FF00FFu;
  a = (a | (a << 4)) & 0x0F0F0F0Fu;
  a = (a | (a << 2)) & 0x33333333u;
  a = (a | (a << 1)) & 0x55555555u;
  return a;
}

// Sort word of source i: (Morton key << 32) | i, or all ones for padding.
__device__ __forceinline__ unsigned long long sort_word(const float* __restrict__ crd_eq,
                                                        int nsrc, int i) {
  unsigned long long v = ~0ull;
  {
    if (i < nsrc) {
      const float x = crd_eq[i], y = crd_eq[(size_t)nsrc + i], z = crd_eq[2 * (size_t)nsrc + i];
      const float n = fabsf(x) + fabsf(y) + fabsf(z);
      float u = n > 0.f ? x / n : 0.f, w = n > 0.f ? y / n : 0.f;
      if (z < 0.f) {
        const float uu = (1.f - fabsf(w)) * (u < 0.f ? -1.f : 1.f);
        const float ww = (1.f - fabsf(u)) * (w < 0.f ? -1.f : 1.f);
        u = uu;
        w = ww;
      }
      // NaN-safe quantisation to [0, 65535]
      const float qu = fminf(fmaxf((u + 1.f) * 32767.5f, 0.f), 65535.f);
      const float qw = fminf(fmaxf((w + 1.f) * 32767.5f, 0.f), 65535.f);
      const uint32_t key = spread16((uint32_t)qu) | (spread16((uint32_t)qw) << 1);
      v = ((unsigned long long)key << 32) | (uint32_t)i;
    }
  }
  return v;
}

__global__ void sort_keys_kernel(const float* __restrict__ crd_eq, int nsrc, int npad,
                                 unsigned long long* __restrict__ kv) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npad; i += gridDim.x * blockDim.x)
    kv[i] = sort_word(crd_eq, nsrc, i);
}

// One compare-exchange pass of the bitonic network (stride j, sequence k).
__global__ void bitonic_global_kernel(unsigned long long* __restrict__ kv, int n, int j, int k) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n / 2; i += gridDim.x * blockDim.x) {
    // i-th pair: lower index has bit j clear
    const int lo = ((i / j) * 2 * j) + (i % j);
    const int hi = lo + j;
    const bool up = (lo & k) == 0;
    const unsigned long long a = kv[lo], b = kv[hi];
    if ((a > b) == up) {
      kv[lo] = b;
      kv[hi] = a;
    }
  }
}

constexpr int kSortTile = 2048;  // elements sorted in shared memory per block

// All passes with stride < kSortTile of sequence lengths k in [k0, k1], in
// shared memory.
__global__ void __launch_bounds__(1024)
bitonic_shared_kernel(unsigned long long* __restrict__ kv, int k0, int k1) {
  __shared__ unsigned long long s[kSortTile];
  const size_t base = (size_t)blockIdx.x * kSortTile;
  s[threadIdx.x] = kv[base + threadIdx.x];
  s[threadIdx.x + 1024] = kv[base + threadIdx.x + 1024];
  __syncthreads();
  for (int k = k0; k <= k1; k <<= 1) {
    for (int j = min(k / 2, kSortTile / 2); j > 0; j >>= 1) {
      const int t = threadIdx.x;
      const int lo = ((t / j) * 2 * j) + (t % j);
      const int hi = lo + j;
      const bool up = ((base + lo) & (size_t)k) == 0;
      const unsigned long long a = s[lo], b = s[hi];
      if ((a > b) == up) {
        s[lo] = b;
        s[hi] = a;
      }
      __syncthreads();
    }
  }
  kv[base + threadIdx.x] = s[threadIdx.x];
  kv[base + threadIdx.x + 1024] = s[threadIdx.x + 1024];
}

__global__ void gather_sorted_kernel(const float* __restrict__ crd_eq, const float* __restrict__ I,
                                     const unsigned long long* __restrict__ kv, int nsrc,
                                     float* __restrict__ crd_s, float* __restrict__ I_s) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nsrc; i += gridDim.x * blockDim.x) {
    const uint32_t src = (uint32_t)(kv[i] & 0xffffffffu);
    crd_s[i] = crd_eq[src];
    crd_s[(size_t)nsrc + i] = crd_eq[(size_t)nsrc + src];
    crd_s[2 * (size_t)nsrc + i] = crd_eq[2 * (size_t)nsrc + src];
    I_s[i] = I[src];
  }
}

// ------------------------------------------------------------ batches ----
// Every simulation of a batch sorted in one set of launches: simulation s
// owns a segment of sort_pad(S_s) words (its own kv buffer), and each pass
// of the network runs within every segment long enough for it, so a
// simulation's order is exactly the one launch_sort_sources gives it alone.
__global__ void sort_keys_batch_kernel(const PrepSim* __restrict__ sims, int nsims,
                                       const long long* __restrict__ pre, long long total) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int si = find_segment(pre, nsims, e);
    const PrepSim& sm = sims[si];
    const int l = (int)(e - __ldg(pre + si));
    sm.kv[l] = sort_word(sm.crd_eq, sm.S, l);
  }
}

__global__ void bitonic_global_batch_kernel(const PrepSim* __restrict__ sims, int nsims,
                                            const long long* __restrict__ pre, long long total,
                                            int j, int k) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int si = find_segment(pre, nsims, e);
    const long long n = 2 * (__ldg(pre + si + 1) - __ldg(pre + si));
    if ((long long)k > n) continue;  // this segment is sorted already
    unsigned long long* kv = sims[si].kv;
    const int i = (int)(e - __ldg(pre + si));
    const int lo = ((i / j) * 2 * j) + (i % j);
    const int hi = lo + j;
    const bool up = (lo & k) == 0;
    const unsigned long long a = kv[lo], b = kv[hi];
    if ((a > b) == up) {
      kv[lo] = b;
      kv[hi] = a;
    }
  }
}

__global__ void __launch_bounds__(1024)
bitonic_shared_batch_kernel(const PrepSim* __restrict__ sims, int nsims,
                            const long long* __restrict__ pre, int k0, int k1) {
  __shared__ unsigned long long s[kSortTile];
  const int si = find_segment(pre, nsims, blockIdx.x);
  const long long n = (long long)kSortTile * (__ldg(pre + si + 1) - __ldg(pre + si));
  if ((long long)k0 > n) return;  // the whole block: one segment
  unsigned long long* kv = sims[si].kv;
  const size_t base = (size_t)(blockIdx.x - __ldg(pre + si)) * kSortTile;
  s[threadIdx.x] = kv[base + threadIdx.x];
  s[threadIdx.x + 1024] = kv[base + threadIdx.x + 1024];
  __syncthreads();
  const int kmax = (int)min((long long)k1, n);
  for (int k = k0; k <= kmax; k <<= 1) {
    for (int j = min(k / 2, kSortTile / 2); j > 0; j >>= 1) {
      const int t = threadIdx.x;
      const int lo = ((t / j) * 2 * j) + (t % j);
      const int hi = lo + j;
      const bool up = ((base + lo) & (size_t)k) == 0;
      const unsigned long long a = s[lo], b = s[hi];
      if ((a > b) == up) {
        s[lo] = b;
        s[hi] = a;
      }
      __syncthreads();
    }
  }
  kv[base + threadIdx.x] = s[threadIdx.x];
  kv[base + threadIdx.x + 1024] = s[threadIdx.x + 1024];
}

__global__ void gather_sorted_batch_kernel(const PrepSim* __restrict__ sims, int nsims,
                                           const long long* __restrict__ pre, long long total) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int si = find_segment(pre, nsims, e);
    const PrepSim& sm = sims[si];
    const int i = (int)(e - __ldg(pre + si));
    if (i >= sm.S) continue;
    const uint32_t src = (uint32_t)(sm.kv[i] & 0xffffffffu);
    const size_t S = (size_t)sm.S;
    sm.crd_s[i] = sm.crd_eq[src];
    sm.crd_s[S + i] = sm.crd_eq[S + src];
    sm.crd_s[2 * S + i] = sm.crd_eq[2 * S + src];
    sm.I_s[i] = sm.I_sky[src];
  }
}

cudaError_t launch_sort_batch(const PrepSim* sims, int nsims, const PrepPre& pre,
                              const PrepTotals& tot, int* launches, cudaStream_t st) {
  int nl = 0;
  const int gk = (int)std::min<long long>((tot.key + 255) / 256, 152 * 16);
  const int gp = (int)std::min<long long>((tot.pair + 255) / 256, 152 * 16);
  sort_keys_batch_kernel<<<gk, 256, 0, st>>>(sims, nsims, pre.key, tot.key);
  ++nl;
  bitonic_shared_batch_kernel<<<(unsigned)tot.tile, 1024, 0, st>>>(sims, nsims, pre.tile, 2,
                                                                    kSortTile);
  ++nl;
  for (int k = 2 * kSortTile; k <= tot.max_key; k <<= 1) {
    for (int j = k / 2; j >= kSortTile; j >>= 1) {
      bitonic_global_batch_kernel<<<gp, 256, 0, st>>>(sims, nsims, pre.pair, tot.pair, j, k);
      ++nl;
    }
    bitonic_shared_batch_kernel<<<(unsigned)tot.tile, 1024, 0, st>>>(sims, nsims, pre.tile, k, k);
    ++nl;
  }
  gather_sorted_batch_kernel<<<gk, 256, 0, st>>>(sims, nsims, pre.key, tot.key);
  ++nl;
  if (launches) *launches = nl;
  return cudaGetLastError();
}

int sort_pad(int nsrc) {
  int n = kSortTile;
  while (n < nsrc) n <<= 1;
  return n;
}

cudaError_t launch_sort_sources(const float* crd_eq, const float* I_sky, int nsrc, void* kv_buf,
                                float* crd_sorted, float* I_sorted, int* launches,
                                cudaStream_t st) {
  const int n = sort_pad(nsrc);
  auto* kv = static_cast<unsigned long long*>(kv_buf);
  const int blocks = std::min(ceil_div(n, 256), 152 * 16);
  int nl = 0;
  sort_keys_kernel<<<blocks, 256, 0, st>>>(crd_eq, nsrc, n, kv);
  ++nl;
  bitonic_shared_kernel<<<n / kSortTile, 1024, 0, st>>>(kv, 2, kSortTile);
  ++nl;
  for (int k = 2 * kSortTile; k <= n; k <<= 1) {
    for (int j = k / 2; j >= kSortTile; j >>= 1) {
      bitonic_global_kernel<<<std::min(ceil_div(n / 2, 256), 152 * 16), 256, 0, st>>>(kv, n, j, k);
      ++nl;
    }
    bitonic_shared_kernel<<<n / kSortTile, 1024, 0, st>>>(kv, k, k);
    ++nl;
  }
  gather_sorted_kernel<<<std::min(ceil_div(nsrc, 256), 152 * 16), 256, 0, st>>>(
      crd_eq, I_sky, kv, nsrc, crd_sorted, I_sorted);
  ++nl;
  if (launches) *launches = nl;
  return cudaGetLastError();
}

}  // namespace hv
