// hv_noalloc.cu -- a visibility entry point that allocates no memory.
//
// Some callers cannot allocate device memory at the point where they want
// visibilities: a real-time pipeline whose device memory is carved up by its
// own pool before it starts and may not grow afterwards, a host framework
// that owns the allocator, or code that runs where cudaMalloc must not be
// called.  hv_vis_gpu_noalloc serves them.  It runs the plain form of the
// hot path (the same kernels as hv_vis_multifreq_device with
// HV_METHOD_PLAIN, precision 1) with all of its working memory -- transposed
// beam, phase coefficients, source records, phasors and split-K partial sums
// -- carved out of one file-scope device array of kNoAllocScratchBytes.
//
// Rules of use
//  - The array exists once per device that loads the library and is held
//    until the process exits.
//  - Host code sees the array's symbol only as a host-side stand-in, so its
//    device address is looked up with cudaGetSymbolAddress, once per device,
//    with that device current, by the first call on that device.  Make that
//    first call before any stream capture.
//  - Every call uses the same array.  Calls whose work overlaps on the GPU
//    (other streams, other host threads) race on it: order them, e.g. on one
//    stream.  Each call writes every word it later reads, so what an earlier
//    call left behind does not matter.
//  - Requests whose working memory exceeds the array are rejected with
//    HV_ERR_ARG and a message naming the bytes needed.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "heravis.h"
#include "hv_internal.cuh"
#include "hv_kernels.h"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;  // 64 MiB
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

void* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

int report(char* buf, size_t len, int code, const char* fmt, ...) {
  if (buf && len) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, len, fmt, ap);
    va_end(ap);
  }
  return code;
}

size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

// The frequency goes to the device as a kernel argument: no copy from host
// memory is queued, so nothing of the call reads the caller's stack later.
__global__ void set_freq_kernel(double* d_freq, double freq) { *d_freq = freq; }

}  // namespace

extern "C" int hv_vis_gpu_noalloc(const void* d_antpos, int nant, double freq,
                                  const void* d_eq2tops, int ntimes, const void* d_crd_eq,
                                  const void* d_I_sky, int nsrc, const void* d_bm_cube,
                                  int beam_px, void* d_vis_out, void* stream, char* errbuf,
                                  size_t errlen) {
  using namespace hv;
  if (errbuf && errlen) errbuf[0] = '\0';
  // the limits of the allocating entry points (check_shapes in hv_api.cu),
  // checked before any size is computed so that no product below overflows
  if (nant < 1 || nant > 65536 || ntimes < 0 || nsrc < 0 || beam_px < 1 || beam_px > 4096)
    return report(errbuf, errlen, HV_ERR_ARG,
                  "bad sizes (nant %d, ntimes %d, nsrc %d, beam_px %d)", nant, ntimes, nsrc,
                  beam_px);
  if (!d_antpos || !d_eq2tops || !d_bm_cube || !d_vis_out || (nsrc > 0 && (!d_crd_eq || !d_I_sky)))
    return report(errbuf, errlen, HV_ERR_ARG, "null array argument");
  if (ntimes == 0) return HV_OK;

  // working memory needed, each region 256-byte aligned
  const int Np = ceil_div(nant, kAntPad) * kAntPad;
  const size_t PP = (size_t)beam_px * beam_px;
  const int S1 = nsrc > 0 ? nsrc : 1;
  const int chunks = ceil_div(S1, kPlainChunk);
  const size_t b_freq = up256(sizeof(double));
  const size_t b_beam = up256(sizeof(float) * PP * Np);
  const size_t b_u = up256(sizeof(Ucoef32) * (size_t)ntimes * Np);
  const size_t b_cnt = up256(sizeof(int) * (size_t)ntimes);
  const size_t b_blk = up256(sizeof(int) * (size_t)prep_blocks(nsrc));
  const size_t b_rec = up256(sizeof(SrcRec32) * (size_t)S1);
  const size_t b_v = up256(sizeof(float2) * (size_t)S1 * Np);
  const size_t b_part = up256(sizeof(float) * (size_t)chunks * 2 * Np * Np);
  const size_t need = b_freq + b_beam + b_u + b_cnt + b_blk + b_rec + b_v + b_part;
  if (need > kNoAllocScratchBytes)
    return report(errbuf, errlen, HV_ERR_ARG,
                  "this request needs %zu bytes of working memory; hv_vis_gpu_noalloc has a "
                  "fixed %zu-byte array (reduce nsrc, nant or beam_px, or use an allocating "
                  "entry point)",
                  need, kNoAllocScratchBytes);

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return report(errbuf, errlen, HV_ERR_CUDA, "cudaGetDevice failed: %s",
                  cudaGetErrorString(e));
  unsigned char* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p)
        return report(errbuf, errlen, HV_ERR_CUDA,
                      "cudaGetSymbolAddress of the working array failed on device %d: %s", dev,
                      cudaGetErrorString(e));
      g_scratch_addr[dev] = p;
    }
    base = static_cast<unsigned char*>(g_scratch_addr[dev]);
  }
  double* d_freq = reinterpret_cast<double*>(base);
  float* beamT = reinterpret_cast<float*>(base + b_freq);
  void* U = base + b_freq + b_beam;
  int* counts = reinterpret_cast<int*>(base + b_freq + b_beam + b_u);
  int* blk = reinterpret_cast<int*>(base + b_freq + b_beam + b_u + b_cnt);
  void* rec = base + b_freq + b_beam + b_u + b_cnt + b_blk;
  void* v = base + b_freq + b_beam + b_u + b_cnt + b_blk + b_rec;
  float* partial = reinterpret_cast<float*>(base + b_freq + b_beam + b_u + b_cnt + b_blk + b_rec + b_v);

  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const float* antpos = static_cast<const float*>(d_antpos);
  const float* e2t = static_cast<const float*>(d_eq2tops);
  const float* crd = static_cast<const float*>(d_crd_eq);
  const float* I = static_cast<const float*>(d_I_sky);
  const size_t NN = (size_t)nant * nant;
#define HV_NA_CK(call)                                                                 \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      return report(errbuf, errlen, HV_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)
  set_freq_kernel<<<1, 1, 0, st>>>(d_freq, freq);
  HV_NA_CK(cudaGetLastError());
  HV_NA_CK(launch_beam_transpose<float>(static_cast<const float*>(d_bm_cube), 1, nant, beam_px,
                                        Np, beamT, st));
  HV_NA_CK(launch_ucoef<float>(antpos, nant, Np, e2t, 0, ntimes, d_freq, 1, U, st));
  for (int t = 0; t < ntimes; ++t) {
    HV_NA_CK(launch_prep<float>(crd, I, nsrc, e2t, t, 1, beam_px, blk, rec, counts + t, st));
    HV_NA_CK(launch_gen_phasors<float>(rec, counts + t, nsrc,
                                       static_cast<const Ucoef32*>(U) + (size_t)t * Np, beamT,
                                       Np, nant, beam_px, v, st));
    HV_NA_CK(launch_herk_plain<float>(v, counts + t, nsrc, Np, partial, st));
    HV_NA_CK(launch_reduce<float>(partial, 0, counts + t, 1, 1, 0, 1, kPlainChunk, Np, nant,
                                  static_cast<float2*>(d_vis_out) + (size_t)t * NN, st));
  }
#undef HV_NA_CK
  return HV_OK;
}
