// hv_plain.cu -- the plain form of the hot path: the reference's method
// (hera_gpu/vis.py:224-250) with its bugs removed.
//
//   gen_phasors : v[s][a] = A_a(l_s, m_s) sqrt(I_s) exp(2 pi i U_a . s)
//                 (InterpolateBeam + MeasEq, vis.py:46-110) written to HBM.
//   herk_plain  : V[a][b] = sum_s v[a,s] conj(v[b,s]) on the upper triangle
//                 only, FP32 (precision 1) or FP64 (precision 2) FMA on the
//                 CUDA cores; the reference runs a full CGEMM/ZGEMM
//                 (vis.py:246-249).  Sources are split into chunks of
//                 kPlainChunk; each chunk's partial sum is stored.
//   reduce      : sums the chunk partials in a fixed order (compensated in
//                 FP32) and writes the full Hermitian matrix, replacing the
//                 host-side sum over chunks of vis.py:258.
#include "hv_internal.cuh"
#include "hv_kernels.h"

namespace hv {

// ------------------------------------------------------------ phasors ----
__device__ __forceinline__ float2 make_phasor(const SrcRec32& r, const Ucoef32& u, float A) {
  return phasor32(r, u, A);
}
__device__ __forceinline__ double2 make_phasor(const SrcRec64& r, const Ucoef64& u, double A) {
  return phasor64(r, u, A);
}

template <typename R>
__global__ void __launch_bounds__(256)
gen_phasors_kernel(const typename Traits<R>::Rec* __restrict__ rec, const int* __restrict__ count,
                   const typename Traits<R>::U* __restrict__ U, const R* __restrict__ beamT,
                   int Np, int nant, int dx, int dy, typename Traits<R>::C* __restrict__ v) {
  using C = typename Traits<R>::C;
  const int n = *count;
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  for (int s = blockIdx.x * wpb + (threadIdx.x >> 5); s < n; s += gridDim.x * wpb) {
    const typename Traits<R>::Rec r = rec[s];
    for (int a = lane; a < Np; a += 32) {
      C val;
      val.x = R(0); val.y = R(0);
      if (a < nant) {
        const R A = beam_bilinear<R>(beamT, Np, a, r, dx, dy);
        val = make_phasor(r, U[a], A);
      }
      v[(size_t)s * Np + a] = val;
    }
  }
}

template <typename R>
cudaError_t launch_gen_phasors(const void* rec, const int* count, int nsrc_max,
                               const void* U, const R* beamT, int Np, int nant, int P,
                               void* v, cudaStream_t st) {
  const int dx = P > 1 ? 1 : 0, dy = P > 1 ? P : 0;
  int blocks = ceil_div(nsrc_max > 0 ? nsrc_max : 1, 8);
  if (blocks > 152 * 64) blocks = 152 * 64;
  gen_phasors_kernel<R><<<blocks, 256, 0, st>>>(
      reinterpret_cast<const typename Traits<R>::Rec*>(rec), count,
      reinterpret_cast<const typename Traits<R>::U*>(U), beamT, Np, nant, dx, dy,
      reinterpret_cast<typename Traits<R>::C*>(v));
  return cudaGetLastError();
}

// ---------------------------------------------------------- SIMT herk ----
constexpr int kHT = 64;   // output tile (antennas) per CTA edge
constexpr int kHK = 16;   // sources per smem stage

__device__ __forceinline__ void decode_upper(int t, int nb, int& I, int& J) {
  I = 0;
  while (t >= nb - I) { t -= nb - I; ++I; }
  J = I + t;
}

template <typename R>
__global__ void __launch_bounds__(256)
herk_plain_kernel(const typename Traits<R>::C* __restrict__ v, const int* __restrict__ count,
                  int Np, R* __restrict__ partial) {
  using C = typename Traits<R>::C;
  const int n = *count;
  const int s0 = blockIdx.y * kPlainChunk;
  if (s0 >= n) return;
  const int s1 = min(s0 + kPlainChunk, n);
  int I, J;
  decode_upper(blockIdx.x, Np / kHT, I, J);

  __shared__ __align__(16) C As[kHK][kHT];
  __shared__ __align__(16) C Bs[kHK][kHT];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  R acc_re[4][4], acc_im[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc_re[i][j] = acc_im[i][j] = R(0);

  const C* vA = v + (size_t)I * kHT;
  const C* vB = v + (size_t)J * kHT;
  C ra[4], rb[4];
  auto gload = [&](int s) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = threadIdx.x + q * 256;
      const int k = idx >> 6, c = idx & 63;
      const bool ok = s + k < s1;
      C z; z.x = R(0); z.y = R(0);
      ra[q] = ok ? vA[(size_t)(s + k) * Np + c] : z;
      rb[q] = ok ? vB[(size_t)(s + k) * Np + c] : z;
    }
  };
  gload(s0);
  for (int s = s0; s < s1; s += kHK) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = threadIdx.x + q * 256;
      As[idx >> 6][idx & 63] = ra[q];
      Bs[idx >> 6][idx & 63] = rb[q];
    }
    __syncthreads();
    if (s + kHK < s1) gload(s + kHK);
    // FP32: each stage's 16 sources are summed from zero and the stage sum
    // is added to the running total, so the total's rounding walks over
    // kPlainChunk / 16 additions instead of kPlainChunk (about 4x less
    // error at the same chunk); FP64 sums straight into the total
    constexpr bool kTwoLevel = sizeof(R) == 4;
    R st_re[4][4], st_im[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        st_re[i][j] = kTwoLevel ? R(0) : acc_re[i][j];
        st_im[i][j] = kTwoLevel ? R(0) : acc_im[i][j];
      }
#pragma unroll
    for (int k = 0; k < kHK; ++k) {
      C a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[k][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[k][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          // v_a conj(v_b) = (ar br + ai bi) + i (ai br - ar bi)
          st_re[i][j] = fma(a[i].x, b[j].x, fma(a[i].y, b[j].y, st_re[i][j]));
          st_im[i][j] = fma(a[i].y, b[j].x, fma(-a[i].x, b[j].y, st_im[i][j]));
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        acc_re[i][j] = kTwoLevel ? acc_re[i][j] + st_re[i][j] : st_re[i][j];
        acc_im[i][j] = kTwoLevel ? acc_im[i][j] + st_im[i][j] : st_im[i][j];
      }
    __syncthreads();
  }
  R* pre = partial + (size_t)blockIdx.y * 2 * Np * Np;
  R* pim = pre + (size_t)Np * Np;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int b = J * kHT + tx * 4 + j;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int a = I * kHT + ty * 4 + i;
      pre[(size_t)b * Np + a] = acc_re[i][j];
      pim[(size_t)b * Np + a] = acc_im[i][j];
    }
  }
}

template <typename R>
cudaError_t launch_herk_plain(const void* v, const int* count, int nsrc_max, int Np,
                              R* partial, cudaStream_t st) {
  const int nb = Np / kHT;
  const int tiles = nb * (nb + 1) / 2;
  const int chunks = nsrc_max > 0 ? ceil_div(nsrc_max, kPlainChunk) : 1;
  dim3 grid(tiles, chunks);
  herk_plain_kernel<R><<<grid, 256, 0, st>>>(
      reinterpret_cast<const typename Traits<R>::C*>(v), count, Np, partial);
  return cudaGetLastError();
}

// ------------------------------------------------------------- reduce ----
struct KahanF {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
};
struct SumD {
  double s = 0.0;
  __device__ __forceinline__ void add(double x) { s += x; }
};
template <typename R> struct Acc;
template <> struct Acc<float> { using type = KahanF; };
template <> struct Acc<double> { using type = SumD; };

// Upper 32 x 32 output tile `tile` of slice sl (block of 256 threads).
template <typename R>
__device__ __forceinline__ void reduce_tile(const R* __restrict__ partial_base,
                                            size_t slice_stride, const int* __restrict__ counts,
                                            int nf, int t0, int ntimes_out, int chunk, int Np,
                                            int nant,
                                            typename Traits<R>::C* __restrict__ out_base,
                                            int tile, int sl,
                                            typename Traits<R>::C (*T)[33]) {
  using C = typename Traits<R>::C;
  const int nbt = ceil_div(nant, 32);
  int A, B;
  decode_upper(tile, nbt, A, B);
  const int tl = sl / nf, f = sl % nf;
  const R* partial = partial_base + (size_t)sl * slice_stride;
  C* out = out_base + ((size_t)f * ntimes_out + t0 + tl) * (size_t)nant * nant;
  const int n = counts[tl];
  const int nk = n > 0 ? ceil_div(n, chunk) : 0;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const size_t plane = (size_t)Np * Np;
  for (int bb = ty; bb < 32; bb += 8) {
    const int a = A * 32 + tx, b = B * 32 + bb;
    typename Acc<R>::type re, im;
    if (a < nant && b < nant) {
      const R* p = partial + (size_t)b * Np + a;
      for (int k = 0; k < nk; ++k) {
        re.add(p[(size_t)k * 2 * plane]);
        im.add(p[(size_t)k * 2 * plane + plane]);
      }
    }
    C val;
    val.x = re.s; val.y = im.s;
    T[bb][tx] = val;
  }
  __syncthreads();
  // out[a][b], b contiguous across the warp
  for (int aa = ty; aa < 32; aa += 8) {
    const int a = A * 32 + aa, b = B * 32 + tx;
    if (a >= nant || b >= nant) continue;
    C val;
    if (A < B || aa <= tx) {
      val = T[tx][aa];
    } else {
      val = T[aa][tx];
      val.y = -val.y;
    }
    if (a == b) val.y = R(0);
    out[(size_t)a * nant + b] = val;
  }
  if (A < B) {
    // mirrored block: out[b][a] = conj(V[a][b]), a contiguous across the warp
    for (int bb = ty; bb < 32; bb += 8) {
      const int a = A * 32 + tx, b = B * 32 + bb;
      if (a >= nant || b >= nant) continue;
      C val = T[bb][tx];
      val.y = -val.y;
      out[(size_t)b * nant + a] = val;
    }
  }
}

template <typename R>
__global__ void __launch_bounds__(256)
reduce_kernel(const R* __restrict__ partial_base, size_t slice_stride,
              const int* __restrict__ counts, int nf, int t0, int ntimes_out, int chunk, int Np,
              int nant, typename Traits<R>::C* __restrict__ out_base) {
  __shared__ typename Traits<R>::C T[32][33];
  reduce_tile<R>(partial_base, slice_stride, counts, nf, t0, ntimes_out, chunk, Np, nant,
                 out_base, blockIdx.x, blockIdx.y, T);
}

// Every simulation of a batch: its split-K chunks reduced into its output.
__global__ void __launch_bounds__(256)
reduce_batch_kernel(const PrepSim* __restrict__ sims, int nsims,
                    const long long* __restrict__ pre) {
  __shared__ float2 T[32][33];
  const int si = find_segment(pre, nsims, blockIdx.x);
  const PrepSim& sm = sims[si];
  const int nbt = ceil_div(sm.nant, 32);
  const int tiles = nbt * (nbt + 1) / 2;
  const int local = (int)(blockIdx.x - __ldg(pre + si));
  const size_t slice = (size_t)ceil_div(sm.S > 0 ? sm.S : 1, sm.chunk) * 2 * sm.Np * sm.Np;
  reduce_tile<float>(sm.partial, slice, sm.counts, sm.F, 0, sm.T, sm.chunk, sm.Np, sm.nant,
                     static_cast<float2*>(sm.out), local % tiles, local / tiles, T);
}

cudaError_t launch_reduce_batch(const PrepSim* sims, int nsims, const PrepPre& pre,
                                const PrepTotals& tot, cudaStream_t st) {
  if (tot.red <= 0) return cudaSuccess;
  reduce_batch_kernel<<<(unsigned)tot.red, 256, 0, st>>>(sims, nsims, pre.red);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_reduce(const R* partial, size_t slice_stride, const int* counts, int nt,
                          int nf, int t0, int ntimes_out, int chunk, int Np, int nant, void* out,
                          cudaStream_t st) {
  const int nbt = ceil_div(nant, 32);
  dim3 grid(nbt * (nbt + 1) / 2, nt * nf);
  reduce_kernel<R><<<grid, 256, 0, st>>>(partial, slice_stride, counts, nf, t0, ntimes_out,
                                         chunk, Np, nant,
                                         reinterpret_cast<typename Traits<R>::C*>(out));
  return cudaGetLastError();
}

template cudaError_t launch_gen_phasors<float>(const void*, const int*, int, const void*, const float*, int, int, int, void*, cudaStream_t);
template cudaError_t launch_gen_phasors<double>(const void*, const int*, int, const void*, const double*, int, int, int, void*, cudaStream_t);
template cudaError_t launch_herk_plain<float>(const void*, const int*, int, int, float*, cudaStream_t);
template cudaError_t launch_herk_plain<double>(const void*, const int*, int, int, double*, cudaStream_t);
template cudaError_t launch_reduce<float>(const float*, size_t, const int*, int, int, int, int, int, int, int, void*, cudaStream_t);
template cudaError_t launch_reduce<double>(const double*, size_t, const int*, int, int, int, int, int, int, int, void*, cudaStream_t);

}  // namespace hv
