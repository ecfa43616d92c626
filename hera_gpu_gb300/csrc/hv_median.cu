// hv_median.cu -- the 2-D median filter of hera_gpu (MedianFilter).
//
// The reference (hera_gpu/median_filter.py:8-365) zero-pads every image by
// half the window on each side (median_filter.py:318), and for each pixel of
// the original image takes the element of rank floor(k0 * k1 / 2) of its
// k0 x k1 window (rows x columns; median_filter.py:223-257, FloydWirth_kth on
// a per-thread copy of the window), one image per stream.
//
// Here one launch covers every image of the call.  3 x 3 windows have their
// own kernel (median3x3_kernel).  Otherwise a block of 8 x 32 output
// pixels stages its window tile -- (8 + k0 - 1) x (32 + k1 - 1) values, the
// zero padding included -- in shared memory as order-preserving 32-bit keys,
// and each thread finds its pixel's rank-k key with no data-dependent
// branches:
//  * windows of up to 81 elements: the k + 1 smallest keys kept sorted in
//    registers, each window key pushed through them by min/max pairs (2 (k+1)
//    integer ops per key);
//  * larger windows: a most-significant-bit-first radix select, 32 counting
//    passes over the keys in shared memory.
// The result is exactly the window's element of that rank (a selection, no
// arithmetic).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>

#include "heravis.h"
#include "hv_kernels.h"

namespace {

constexpr int kMfCols = 32;  // output columns per block (a warp's lanes)
constexpr int kMfRows = 8;   // output rows per block
constexpr int kMfSmemLimit = 200 * 1024;

// Keys that order like the floats: negative values have every bit flipped,
// the others the sign bit set.
__device__ __forceinline__ uint32_t mf_key(float x) {
  const uint32_t u = __float_as_uint(x);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float mf_value(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__device__ __forceinline__ uint32_t med3u(uint32_t a, uint32_t b, uint32_t c) {
  return max(min(a, b), min(max(a, b), c));
}

// Median of an H x W window (H W odd) by forgetful selection: the first
// n / 2 + 2 keys (n = H W) are held in registers; for each further key the
// buffer's maximum is bubbled to its top and its minimum to its bottom, both
// are dropped (neither can be the median: each has more than n / 2 keys on
// its other side, counting the keys dropped before) and the new key takes
// the maximum's place.  The median of the three keys left is the window's.
// About n^2 / 2 min/max operations, against 2 (n / 2 + 1) n for the
// register insertion below.
template <int H, int W>
__device__ __forceinline__ uint32_t forgetful_median(const uint32_t* win, int tw) {
  constexpr int N = H * W, R0 = N / 2 + 2;
  static_assert(N % 2 == 1 && N >= 3, "odd windows of at least 3 keys");
  uint32_t a[R0];
#pragma unroll
  for (int e = 0; e < R0; ++e) a[e] = win[(e / W) * tw + e % W];
#pragma unroll
  for (int e = R0; e < N; ++e) {
    const int lo = e - R0;  // the buffer is a[lo .. R0 - 1]
#pragma unroll
    for (int i = lo; i < R0 - 1; ++i) {
      const uint32_t x = min(a[i], a[i + 1]);
      a[i + 1] = max(a[i], a[i + 1]);
      a[i] = x;
    }
#pragma unroll
    for (int i = R0 - 2; i > lo; --i) {
      const uint32_t x = min(a[i - 1], a[i]);
      a[i] = max(a[i - 1], a[i]);
      a[i - 1] = x;
    }
    a[R0 - 1] = win[(e / W) * tw + e % W];
  }
  return med3u(a[R0 - 3], a[R0 - 2], a[R0 - 1]);
}

// grid (ceil(cols / 32), ceil(rows / 8), nimg), block (32, 8); dynamic shared
// memory (8 + k0 - 1) * (32 + k1 - 1) keys.  H > 0: an H x W window (k0 = H,
// k1 = W) by forgetful selection; else K > 0: windows of at most 2 K - 1
// elements select with K registers; K == 0: radix select.
template <int K, int H = 0, int W = 0>
__global__ void __launch_bounds__(kMfCols * kMfRows)
median_filter_kernel(const float* __restrict__ in, float* __restrict__ out, int rows, int cols,
                     int k0, int k1) {
  extern __shared__ uint32_t tile[];
  const int tw = kMfCols + k1 - 1, th = kMfRows + k0 - 1;
  // tile origin in image coordinates (the window of pixel (r, c) starts at
  // (r - k0 / 2, c - k1 / 2), as the reference's padded image)
  const int r0 = (int)blockIdx.y * kMfRows - k0 / 2;
  const int c0 = (int)blockIdx.x * kMfCols - k1 / 2;
  const size_t plane = (size_t)rows * cols;
  const float* img = in + (size_t)blockIdx.z * plane;
  for (int i = (int)(threadIdx.y * kMfCols + threadIdx.x); i < tw * th; i += kMfCols * kMfRows) {
    const int r = r0 + i / tw, c = c0 + i % tw;
    const float v = (r >= 0 && r < rows && c >= 0 && c < cols) ? img[(size_t)r * cols + c] : 0.f;
    tile[i] = mf_key(v);
  }
  __syncthreads();
  const int r = (int)(blockIdx.y * kMfRows + threadIdx.y), c = (int)(blockIdx.x * kMfCols + threadIdx.x);
  if (r >= rows || c >= cols) return;
  const uint32_t* win = tile + threadIdx.y * tw + threadIdx.x;
  const int rank = (k0 * k1) / 2;
  if constexpr (H > 0) {
    out[(size_t)blockIdx.z * plane + (size_t)r * cols + c] = mf_value(forgetful_median<H, W>(win, tw));
    return;
  }
  if (K > 0) {
    // s[0..K) holds the smallest keys seen so far, ascending; a new key
    // sinks to its place and the largest falls out
    uint32_t sm[K > 0 ? K : 1];
#pragma unroll
    for (int q = 0; q < K; ++q) sm[q] = 0xffffffffu;
    for (int i = 0; i < k0; ++i) {
      const uint32_t* row = win + i * tw;
      for (int j = 0; j < k1; ++j) {
        uint32_t v = row[j];
#pragma unroll
        for (int q = 0; q < K; ++q) {
          const uint32_t lo = min(sm[q], v);
          v = max(sm[q], v);
          sm[q] = lo;
        }
      }
    }
    // rank <= K - 1: pick sm[rank] without dynamic indexing
    uint32_t key = sm[0];
#pragma unroll
    for (int q = 1; q < K; ++q) key = q == rank ? sm[q] : key;
    out[(size_t)blockIdx.z * plane + (size_t)r * cols + c] = mf_value(key);
    return;
  }
  // radix select of the rank-k key, most significant bit first: at bit b
  // the candidates share `prefix` above b; count those with bit b clear
  int left = rank;
  uint32_t prefix = 0;
#pragma unroll 1
  for (int b = 31; b >= 0; --b) {
    const uint32_t bit = 1u << b;
    const uint32_t mask = ~(bit - 1u);  // bits b..31
    int cnt = 0;
#pragma unroll 1
    for (int i = 0; i < k0; ++i) {
      const uint32_t* row = win + i * tw;
#pragma unroll 4
      for (int j = 0; j < k1; ++j) cnt += (row[j] & mask) == prefix;
    }
    if (left >= cnt) {
      left -= cnt;
      prefix |= bit;
    }
  }
  out[(size_t)blockIdx.z * plane + (size_t)r * cols + c] = mf_value(prefix);
}

// The 3 x 3 window (the reference's default): with each window column
// sorted into (lo, mid, hi), the median of the nine is
// med3(max of the three lo, med3 of the three mid, min of the three hi), an
// exact selection.  A block of 128 x 16 outputs stages its 130 x 18 tile of
// keys (rows padded to 132 keys, 16-byte aligned); each thread takes 4
// columns x 2 rows of outputs, so it sorts 6 columns of 4 input rows once
// (the middle pair shared by both output rows) and reads them with one
// 128-bit and one 64-bit load per row.
constexpr int kM3Cols = 128, kM3Rows = 16, kM3Pitch = 132;

// vec: rows of the output start 16-byte aligned (cols % 4 == 0 and an
// aligned base), so whole groups of 4 are stored as one float4.
__global__ void __launch_bounds__(256) median3x3_kernel(const float* __restrict__ in,
                                                        float* __restrict__ out, int rows,
                                                        int cols, bool vec) {
  __shared__ __align__(16) uint32_t tile[(kM3Rows + 2) * kM3Pitch];
  const int r0 = (int)blockIdx.y * kM3Rows - 1, c0 = (int)blockIdx.x * kM3Cols - 1;
  const size_t plane = (size_t)rows * cols;
  const float* img = in + (size_t)blockIdx.z * plane;
  const int tid = (int)(threadIdx.y * 32 + threadIdx.x);
  for (int i = tid; i < (kM3Rows + 2) * (kM3Cols + 2); i += 256) {
    const int tr = i / (kM3Cols + 2), tc = i - tr * (kM3Cols + 2);
    const int r = r0 + tr, c = c0 + tc;
    const float v = (r >= 0 && r < rows && c >= 0 && c < cols) ? img[(size_t)r * cols + c] : 0.f;
    tile[tr * kM3Pitch + tc] = mf_key(v);
  }
  __syncthreads();
  const int tx = (int)threadIdx.x, ty = (int)threadIdx.y;
  uint32_t k[4][6];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const uint32_t* row = tile + (2 * ty + i) * kM3Pitch + 4 * tx;
    const uint4 a = *reinterpret_cast<const uint4*>(row);
    const uint2 b = *reinterpret_cast<const uint2*>(row + 4);
    k[i][0] = a.x;
    k[i][1] = a.y;
    k[i][2] = a.z;
    k[i][3] = a.w;
    k[i][4] = b.x;
    k[i][5] = b.y;
  }
  // sorted columns of input rows 0-2 (output row 0) and 1-3 (output row 1)
  uint32_t lo[2][6], md[2][6], hi[2][6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const uint32_t p = min(k[1][j], k[2][j]), q = max(k[1][j], k[2][j]);
#pragma unroll
    for (int o = 0; o < 2; ++o) {
      const uint32_t x = k[o ? 3 : 0][j];
      lo[o][j] = min(p, x);
      hi[o][j] = max(q, x);
      md[o][j] = max(p, min(q, x));
    }
  }
  const int c = (int)blockIdx.x * kM3Cols + 4 * tx;
#pragma unroll
  for (int o = 0; o < 2; ++o) {
    const int r = (int)blockIdx.y * kM3Rows + 2 * ty + o;
    uint32_t v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t mx = max(max(lo[o][q], lo[o][q + 1]), lo[o][q + 2]);
      const uint32_t mn = min(min(hi[o][q], hi[o][q + 1]), hi[o][q + 2]);
      v[q] = med3u(mx, med3u(md[o][q], md[o][q + 1], md[o][q + 2]), mn);
    }
    if (r < rows) {
      float* dst = out + (size_t)blockIdx.z * plane + (size_t)r * cols + c;
      if (vec && c + 3 < cols) {
        *reinterpret_cast<float4*>(dst) =
            make_float4(mf_value(v[0]), mf_value(v[1]), mf_value(v[2]), mf_value(v[3]));
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (c + q < cols) dst[q] = mf_value(v[q]);
      }
    }
  }
}

int check_args(hv_context* ctx, int nimg, int rows, int cols, int k0, int k1, size_t* smem) {
  char msg[256];
  if (nimg < 0 || rows < 0 || cols < 0 || k0 < 1 || k1 < 1 || nimg > 65535 ||
      (long long)rows > 65535LL * kMfRows) {
    snprintf(msg, sizeof msg, "median filter: bad sizes (images %d, %d x %d, window %d x %d)",
             nimg, rows, cols, k0, k1);
    if (ctx) hv_context_set_error(ctx, msg);
    return HV_ERR_ARG;
  }
  *smem = sizeof(uint32_t) * (size_t)(kMfRows + k0 - 1) * (kMfCols + k1 - 1);
  if (*smem > (size_t)kMfSmemLimit) {
    snprintf(msg, sizeof msg, "median filter: a %d x %d window needs %zu bytes of shared memory "
             "per block (at most %d)", k0, k1, *smem, kMfSmemLimit);
    if (ctx) hv_context_set_error(ctx, msg);
    return HV_ERR_ARG;
  }
  return HV_OK;
}

int launch(hv_context* ctx, const float* d_in, float* d_out, int nimg, int rows, int cols, int k0,
           int k1, cudaStream_t st) {
  size_t smem = 0;
  int r = check_args(ctx, nimg, rows, cols, k0, k1, &smem);
  if (r != HV_OK) return r;
  if ((size_t)nimg * rows * cols == 0) return HV_OK;
  static bool configured = false;
  if (!configured) {
    for (const void* k : {reinterpret_cast<const void*>(median_filter_kernel<0>),
                          reinterpret_cast<const void*>(median_filter_kernel<1>),
                          reinterpret_cast<const void*>(median_filter_kernel<5>),
                          reinterpret_cast<const void*>(median_filter_kernel<13>),
                          reinterpret_cast<const void*>(median_filter_kernel<25>),
                          reinterpret_cast<const void*>(median_filter_kernel<41>),
                          reinterpret_cast<const void*>(median_filter_kernel<0, 5, 5>),
                          reinterpret_cast<const void*>(median_filter_kernel<0, 7, 7>),
                          reinterpret_cast<const void*>(median_filter_kernel<0, 9, 9>),
                          reinterpret_cast<const void*>(median_filter_kernel<0, 9, 5>),
                          reinterpret_cast<const void*>(median_filter_kernel<0, 5, 9>)})
      if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kMfSmemLimit) !=
          cudaSuccess)
        return HV_ERR_CUDA;
    configured = true;
  }
  const dim3 grid((cols + kMfCols - 1) / kMfCols, (rows + kMfRows - 1) / kMfRows, nimg);
  const dim3 block(kMfCols, kMfRows);
  const int n = k0 * k1;  // the register forms need n / 2 + 1 <= K
  if (k0 == 3 && k1 == 3)
    median3x3_kernel<<<dim3((cols + kM3Cols - 1) / kM3Cols, (rows + kM3Rows - 1) / kM3Rows, nimg),
                       dim3(32, 8), 0, st>>>(d_in, d_out, rows, cols,
                                             (cols & 3) == 0 &&
                                                 (reinterpret_cast<uintptr_t>(d_out) & 15) == 0);
  else if (k0 == 5 && k1 == 5)
    median_filter_kernel<0, 5, 5><<<grid, block, smem, st>>>(d_in, d_out, rows, cols, k0, k1);
  else if (k0 == 7 && k1 == 7)
    median_filter_kernel<0, 7, 7><<<grid, block, smem, st>>>(d_in, d_out, rows, cols, k0, k1);
  else if (k0 == 9 && k1 == 9)
    median_filter_kernel<0, 9, 9><<<grid, block, smem, st>>>(d_in, d_out, rows, cols, k0, k1);
  else if (k0 == 9 && k1 == 5)
    median_filter_kernel<0, 9, 5><<<grid, block, smem, st>>>(d_in, d_out, rows, cols, k0, k1);
  else if (k0 == 5 && k1 == 9)
    median_filter_kernel<0, 5, 9><<<grid, block, smem, st>>>(d_in, d_out, rows, cols, k0, k1);
  else if (n <= 1) median_filter_kernel<1><<<grid, block, smem, st>>>(d_in, d_out, rows, cols, k0, k1);
  else if (n <= 9) median_filter_kernel<5><<<grid, block, smem, st>>>(d_in, d_out, rows, cols, k0, k1);
  else if (n <= 25) median_filter_kernel<13><<<grid, block, smem, st>>>(d_in, d_out, rows, cols, k0, k1);
  else if (n <= 49) median_filter_kernel<25><<<grid, block, smem, st>>>(d_in, d_out, rows, cols, k0, k1);
  else if (n <= 81) median_filter_kernel<41><<<grid, block, smem, st>>>(d_in, d_out, rows, cols, k0, k1);
  else median_filter_kernel<0><<<grid, block, smem, st>>>(d_in, d_out, rows, cols, k0, k1);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    if (ctx) hv_context_set_error(ctx, cudaGetErrorString(e));
    return HV_ERR_CUDA;
  }
  hv_context_add_launches(ctx, 1);
  return HV_OK;
}

}  // namespace

extern "C" {

int hv_median_filter_device(hv_context* ctx, const float* d_in, float* d_out, int nimg, int rows,
                            int cols, int k0, int k1, void* stream) {
  const bool empty = nimg <= 0 || rows <= 0 || cols <= 0;
  if (!ctx || (!empty && (!d_in || !d_out))) return HV_ERR_ARG;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : hv_context_stream(ctx);
  return launch(ctx, d_in, d_out, nimg, rows, cols, k0, k1, st);
}

int hv_median_filter(hv_context* ctx, const float* in, float* out, int nimg, int rows, int cols,
                     int k0, int k1) {
  if (!ctx) return HV_ERR_ARG;
  size_t smem = 0;
  int r = check_args(ctx, nimg, rows, cols, k0, k1, &smem);
  if (r != HV_OK) return r;
  const size_t bytes = sizeof(float) * (size_t)nimg * rows * cols;
  if (bytes == 0) return HV_OK;
  if (!in || !out) return HV_ERR_ARG;
  cudaStream_t st = hv_context_stream(ctx);
  void *d_in = nullptr, *d_out = nullptr;
  if (cudaMallocAsync(&d_in, bytes, st) != cudaSuccess ||
      cudaMallocAsync(&d_out, bytes, st) != cudaSuccess) {
    cudaGetLastError();
    if (d_in) cudaFreeAsync(d_in, st);
    hv_context_set_error(ctx, "median filter: device allocation failed");
    return HV_ERR_OOM;
  }
  r = HV_OK;
  if (cudaMemcpyAsync(d_in, in, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess) r = HV_ERR_CUDA;
  if (r == HV_OK)
    r = launch(ctx, static_cast<const float*>(d_in), static_cast<float*>(d_out), nimg, rows,
               cols, k0, k1, st);
  if (r == HV_OK &&
      cudaMemcpyAsync(out, d_out, bytes, cudaMemcpyDeviceToHost, st) != cudaSuccess)
    r = HV_ERR_CUDA;
  cudaFreeAsync(d_in, st);
  cudaFreeAsync(d_out, st);
  if (cudaStreamSynchronize(st) != cudaSuccess && r == HV_OK) r = HV_ERR_CUDA;
  return r;
}

}  // extern "C"
