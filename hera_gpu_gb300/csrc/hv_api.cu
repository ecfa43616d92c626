// hv_api.cu -- the C ABI of libheravis.so (include/heravis.h) and the host
// orchestration behind it.
//
// Per call (reference hera_gpu/vis.py:144-262, restructured):
//   1. beam cubes -> [freq][pixel][antenna] (one kernel for all frequencies)
//   2. phase coefficients U for every (time, frequency, antenna)
//   3. per time: rotate + horizon-cut + beam corners for all sources (once,
//      shared by every frequency), then per frequency the visibility kernels
//      and an on-device reduction straight into the output slice.
// Everything is ordered on one stream; no host synchronisation inside the
// loops (the reference synchronises and sums on the host every time step,
// vis.py:257-258).
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "heravis.h"
#include "hv_internal.cuh"
#include "hv_kernels.h"

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};
struct HostBuf {
  void* p = nullptr;
  size_t cap = 0;
};

}  // namespace

struct hv_context {
  int device = 0;
  int num_sms = 0;
  int cc_major = 0, cc_minor = 0;
  cudaStream_t stream = nullptr;
  // a fused launch of one simulation shared between its cluster kernel and a
  // one-CTA kernel on the SMs no cluster fits on (launch_tc_batch)
  hv::TcShare share{};
  // end of a device-API call made on a caller's stream: the context's stream
  // waits on it, so hv_sync and the error-flag read come after that work
  cudaEvent_t joined = nullptr;
  size_t budget = 0;  // 0 = unlimited
  size_t held = 0;
  std::string err;
  uint64_t launches = 0;
  int* d_err = nullptr;  // device-side error flag (bounded waits)
  unsigned long long* d_claim = nullptr;  // item-claim counter of the fused launches
  // profiling of the visibility-product kernels
  bool profiling = false;
  // device-side wait limit of the fused kernel (0: its default) and fault
  // injection (hv_set_wait_limit)
  uint64_t wait_ns = 0;
  int stall = 0;
  // launch shape of the fused kernel (hv_set_tuning; zeros = defaults)
  hv::TcTune tune{};
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_events;
  // staging of host-API inputs / outputs
  DevBuf in_antpos, in_eq2tops, in_crd, in_I, in_bm, out_vis;
  // workspace
  DevBuf freqs, beamT, ucoef, rec, counts, blkcounts, v, partial, tcgroups;
  DevBuf umax, sortkv, crd_sorted, I_sorted, tctable, pixmax, sbound;
  HostBuf tctable_h;  // page-locked staging of the fused kernel's simulation table
  // page-locked blocks given back by destroyed batches, kept for the next
  // ones: freeing page-locked memory waits for the whole device
  std::vector<std::pair<void*, size_t>> host_pool;
};

namespace {

int fail(hv_context* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

#define HV_CK(call)                                                              \
  do {                                                                           \
    cudaError_t e_ = (call);                                                     \
    if (e_ != cudaSuccess)                                                       \
      return fail(ctx, HV_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

#define HV_LAUNCH(n, call)     \
  do {                         \
    HV_CK(call);               \
    ctx->launches += (n);      \
  } while (0)

// A launch of a visibility-product kernel, bracketed by events when profiling.
#define HV_LAUNCH_TIMED(call, st)                                   \
  do {                                                              \
    cudaEvent_t e0_ = nullptr, e1_ = nullptr;                       \
    if (ctx->profiling) {                                           \
      HV_CK(cudaEventCreate(&e0_));                                 \
      HV_CK(cudaEventCreate(&e1_));                                 \
      HV_CK(cudaEventRecord(e0_, (st)));                            \
    }                                                               \
    HV_LAUNCH(1, call);                                             \
    if (ctx->profiling) {                                           \
      HV_CK(cudaEventRecord(e1_, (st)));                            \
      ctx->prof_events.emplace_back(e0_, e1_);                      \
    }                                                               \
  } while (0)

int ensure(hv_context* ctx, DevBuf& b, size_t bytes) {
  if (bytes == 0) bytes = 256;
  if (b.cap >= bytes) return HV_OK;
  // the old buffer may still be read by queued work (on any stream)
  HV_CK(cudaDeviceSynchronize());
  if (b.p) {
    HV_CK(cudaFree(b.p));
    ctx->held -= b.cap;
    b.p = nullptr;
    b.cap = 0;
  }
  size_t want = bytes + bytes / 8;  // slack against regrowth
  if (ctx->budget && ctx->held + want > ctx->budget) want = bytes;
  if (ctx->budget && ctx->held + want > ctx->budget)
    return fail(ctx, HV_ERR_OOM, "workspace of %zu bytes exceeds the HBM budget (%zu held of %zu)",
                want, ctx->held, ctx->budget);
  cudaError_t e = cudaMalloc(&b.p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    b.p = nullptr;
    return fail(ctx, HV_ERR_OOM, "cudaMalloc(%zu) failed: %s", want, cudaGetErrorString(e));
  }
  b.cap = want;
  ctx->held += want;
  return HV_OK;
}

// Page-locked host buffer that stays valid for the copies queued from it.
int ensure_host(hv_context* ctx, HostBuf& b, size_t bytes) {
  if (b.cap >= bytes) return HV_OK;
  HV_CK(cudaDeviceSynchronize());
  if (b.p) HV_CK(cudaFreeHost(b.p));
  b.p = nullptr;
  b.cap = 0;
  HV_CK(cudaHostAlloc(&b.p, bytes, cudaHostAllocDefault));
  b.cap = bytes;
  return HV_OK;
}

#define HV_HOST_ENSURE(buf, bytes)               \
  do {                                           \
    int r_ = ensure_host(ctx, (buf), (bytes));   \
    if (r_ != HV_OK) return r_;                  \
  } while (0)

#define HV_ENSURE(buf, bytes)                 \
  do {                                        \
    int r_ = ensure(ctx, (buf), (bytes));     \
    if (r_ != HV_OK) return r_;               \
  } while (0)

void release(hv_context* ctx, DevBuf& b) {
  if (b.p) cudaFree(b.p);
  ctx->held -= b.cap;
  b.p = nullptr;
  b.cap = 0;
}

int check_shapes(hv_context* ctx, int precision, int method, int nant, int nfreq,
                 int ntimes, int nsrc, int P) {
  if (precision != 1 && precision != 2)
    return fail(ctx, HV_ERR_ARG, "precision must be 1 or 2 (got %d)", precision);
  if (method < HV_METHOD_AUTO || method > HV_METHOD_TC_FP16)
    return fail(ctx, HV_ERR_ARG, "unknown method %d", method);
  if (precision == 2 && (method == HV_METHOD_TC_BF16 || method == HV_METHOD_TC_FP16))
    return fail(ctx, HV_ERR_ARG,
                "the tensor-core methods compute in FP32 with BF16 or FP16/FP8 operands; use "
                "precision 1");
  if (nant < 1) return fail(ctx, HV_ERR_ARG, "nant must be >= 1 (got %d)", nant);
  if (nant > 65536) return fail(ctx, HV_ERR_ARG, "nant %d too large", nant);
  if (nfreq < 1) return fail(ctx, HV_ERR_ARG, "nfreq must be >= 1 (got %d)", nfreq);
  if (ntimes < 0) return fail(ctx, HV_ERR_ARG, "ntimes must be >= 0 (got %d)", ntimes);
  if (nsrc < 0) return fail(ctx, HV_ERR_ARG, "nsrc must be >= 0 (got %d)", nsrc);
  // (time, frequency) slices are counted in int by the kernels
  if ((long long)ntimes * nfreq > 0x7fffffffLL)
    return fail(ctx, HV_ERR_ARG, "ntimes x nfreq = %lld slices exceeds 2^31 - 1",
                (long long)ntimes * nfreq);
  if (P < 1 || P > 4096) return fail(ctx, HV_ERR_ARG, "beam_px must be in [1, 4096] (got %d)", P);
  return HV_OK;
}

// Workspace caps for the tensor-core path: split-K partial sums and source
// records of one batch of times.
constexpr size_t kTcPartialCap = size_t(6) << 30;
constexpr size_t kTcRecCap = size_t(4) << 30;

template <typename R>
int run_device(hv_context* ctx, int method, const R* antpos, int nant, const double* freqs,
               int nfreq, const R* eq2tops, int ntimes, const R* crd_eq, const R* I_sky,
               int nsrc, const R* bm, int P, void* out, cudaStream_t st) {
  using namespace hv;
  using C = typename Traits<R>::C;
  using U = typename Traits<R>::U;
  using Rec = typename Traits<R>::Rec;
  if (ntimes == 0) return HV_OK;
  const int Np = ceil_div(nant, kAntPad) * kAntPad;
  const size_t PP = (size_t)P * P;
  const bool tc = (method == HV_METHOD_TC_BF16) || (method == HV_METHOD_TC_FP16) ||
                  (method == HV_METHOD_AUTO && sizeof(R) == 4);
  const int form = method == HV_METHOD_TC_FP16 ? 1 : 0;

  HV_ENSURE(ctx->freqs, sizeof(double) * nfreq);
  HV_CK(cudaMemcpyAsync(ctx->freqs.p, freqs, sizeof(double) * nfreq, cudaMemcpyHostToDevice, st));
  HV_ENSURE(ctx->beamT, sizeof(R) * nfreq * PP * Np);
  HV_ENSURE(ctx->ucoef, sizeof(U) * (size_t)ntimes * nfreq * Np);
  HV_ENSURE(ctx->counts, sizeof(int) * (size_t)ntimes);
  R* beamT = static_cast<R*>(ctx->beamT.p);
  HV_LAUNCH(1, launch_beam_transpose<R>(bm, nfreq, nant, P, Np, beamT, st));
  HV_LAUNCH(1, launch_ucoef<R>(antpos, nant, Np, eq2tops, 0, ntimes,
                               static_cast<const double*>(ctx->freqs.p), nfreq, ctx->ucoef.p, st));
  int* counts = static_cast<int*>(ctx->counts.p);
  const size_t NN = (size_t)nant * nant;
  const int S1 = nsrc > 0 ? nsrc : 1;

  if (tc) {
    if constexpr (sizeof(R) == 4) {
      // group table of the 128-antenna block pairs
      const size_t gbytes = tc_group_table_bytes(nant);
      std::string host(gbytes, '\0');
      const int ngroups = tc_fill_group_table(nant, &host[0]);
      HV_ENSURE(ctx->tcgroups, gbytes);
      HV_CK(cudaMemcpyAsync(ctx->tcgroups.p, host.data(), gbytes, cudaMemcpyHostToDevice, st));
      // batch of times per launch, bounded by the partial-sum and record caps
      int ntb = ntimes, chunk = 0;
      size_t slice_floats = 0;
      for (;;) {
        chunk = tc_chunk_sources(S1, ntb * nfreq, ngroups, ctx->num_sms);
        slice_floats = tc_partial_floats(Np, S1, 1, chunk);
        const size_t pbytes = sizeof(float) * slice_floats * (size_t)ntb * nfreq;
        const size_t rbytes = sizeof(Rec) * (size_t)ntb * (((size_t)S1 + 31) / 32 * 32);
        if (ntb == 1 || (pbytes <= kTcPartialCap && rbytes <= kTcRecCap)) break;
        ntb = (ntb + 1) / 2;
      }
      HV_ENSURE(ctx->partial, sizeof(float) * slice_floats * (size_t)ntb * nfreq);
      const size_t rec_stride = ((size_t)S1 + 31) / 32 * 32;  // whole stages per time
      HV_ENSURE(ctx->rec, sizeof(Rec) * (size_t)ntb * rec_stride);
      HV_ENSURE(ctx->blkcounts, sizeof(int) * (size_t)prep_blocks(nsrc) * ntb);
      // per-slice bound of |U|_1, and the catalogue in spatial order
      HV_ENSURE(ctx->umax, sizeof(float) * (size_t)ntimes * nfreq);
      HV_LAUNCH(1, launch_ubound(ctx->ucoef.p, ntimes * nfreq, Np,
                                 static_cast<float*>(ctx->umax.p), st));
      // FP16 + FP8 form: the beam's largest value per pixel, for the slices'
      // scales
      if (form == 1) {
        HV_ENSURE(ctx->pixmax, sizeof(float) * (size_t)nfreq * PP);
        HV_ENSURE(ctx->sbound, sizeof(float) * (size_t)ntimes * nfreq);
        HV_LAUNCH(1, launch_beam_pixmax(reinterpret_cast<const float*>(beamT), nfreq, P, Np,
                                        static_cast<float*>(ctx->pixmax.p), st));
      }
      const R* crd_use = crd_eq;
      const R* I_use = I_sky;
      if (nsrc > 0) {
        HV_ENSURE(ctx->sortkv, sizeof(unsigned long long) * (size_t)sort_pad(nsrc));
        HV_ENSURE(ctx->crd_sorted, sizeof(float) * 3 * (size_t)nsrc);
        HV_ENSURE(ctx->I_sorted, sizeof(float) * (size_t)nsrc);
        int nl = 0;
        HV_CK(launch_sort_sources(reinterpret_cast<const float*>(crd_eq),
                                  reinterpret_cast<const float*>(I_sky), nsrc, ctx->sortkv.p,
                                  static_cast<float*>(ctx->crd_sorted.p),
                                  static_cast<float*>(ctx->I_sorted.p), &nl, st));
        ctx->launches += nl;
        crd_use = static_cast<const R*>(ctx->crd_sorted.p);
        I_use = static_cast<const R*>(ctx->I_sorted.p);
      }
      for (int t0 = 0; t0 < ntimes; t0 += ntb) {
        const int nt = std::min(ntb, ntimes - t0);
        HV_LAUNCH(2, launch_prep_strided<R>(crd_use, I_use, nsrc, eq2tops, t0, nt, P,
                                            static_cast<int*>(ctx->blkcounts.p), ctx->rec.p,
                                            rec_stride, counts + t0, st));
        HV_LAUNCH(1, launch_tc_relative(ctx->rec.p, rec_stride, counts + t0, nt, nsrc, st));
        float* sbound = nullptr;
        if (form == 1) {
          sbound = static_cast<float*>(ctx->sbound.p) + (size_t)t0 * nfreq;
          HV_LAUNCH(1, launch_slice_bound(ctx->rec.p, rec_stride, counts + t0, nt, nsrc,
                                          static_cast<const float*>(ctx->pixmax.p), nfreq, P,
                                          sbound, st));
        }
        TcSimDesc L{};
        L.sbound = sbound;
        L.form = form;
        L.tune = ctx->tune;
        L.counts = counts + t0;
        L.U = static_cast<const U*>(ctx->ucoef.p) + (size_t)t0 * nfreq * Np;
        L.beamT = reinterpret_cast<const float*>(beamT);
        L.umax = static_cast<const float*>(ctx->umax.p) + (size_t)t0 * nfreq;
        L.partial = static_cast<float*>(ctx->partial.p);
        L.groups = ctx->tcgroups.p;
        L.ngroups = ngroups;
        L.max_slots = tc_max_slots(nant);
        L.rec_row0 = 0;
        L.rec_stride = (int)rec_stride;
        L.nt = nt;
        L.nf = nfreq;
        L.Np = Np;
        L.nant = nant;
        L.P = P;
        L.nsrc = nsrc;
        L.chunk = chunk;
        HV_ENSURE(ctx->tctable, tc_sim_table_bytes(1));
        HV_HOST_ENSURE(ctx->tctable_h, tc_sim_table_bytes(1));
        if (nsrc > 0)
          HV_LAUNCH_TIMED(launch_tc_batch(&L, 1, ctx->rec.p, (long long)nt * rec_stride,
                                          ctx->tctable.p, ctx->tctable_h.p, ctx->d_err,
                                          ctx->d_claim, ctx->num_sms, st, ctx->wait_ns,
                                          ctx->stall, &ctx->share),
                          st);
        if (nsrc > 0 && ctx->share.launched > 1) ctx->launches += ctx->share.launched - 1;
        HV_LAUNCH(1, launch_reduce<float>(static_cast<float*>(ctx->partial.p), slice_floats,
                                          counts + t0, nt, nfreq, t0, ntimes, chunk, Np, nant,
                                          out, st));
      }
    }
    return HV_OK;
  }

  // plain form: one time at a time, one frequency at a time
  const int chunks = ceil_div(S1, kPlainChunk);
  HV_ENSURE(ctx->partial, sizeof(R) * (size_t)chunks * 2 * Np * Np);
  HV_ENSURE(ctx->v, sizeof(C) * (size_t)S1 * Np);
  HV_ENSURE(ctx->rec, sizeof(Rec) * (size_t)S1);
  HV_ENSURE(ctx->blkcounts, sizeof(int) * (size_t)prep_blocks(nsrc));
  for (int t = 0; t < ntimes; ++t) {
    HV_LAUNCH(2, launch_prep<R>(crd_eq, I_sky, nsrc, eq2tops, t, 1, P,
                                static_cast<int*>(ctx->blkcounts.p), ctx->rec.p, counts + t, st));
    const U* Ut = static_cast<const U*>(ctx->ucoef.p) + (size_t)t * nfreq * Np;
    for (int f = 0; f < nfreq; ++f) {
      C* o = static_cast<C*>(out) + ((size_t)f * ntimes + t) * NN;
      HV_LAUNCH(1, launch_gen_phasors<R>(ctx->rec.p, counts + t, nsrc, Ut + (size_t)f * Np,
                                         beamT + (size_t)f * PP * Np, Np, nant, P, ctx->v.p, st));
      HV_LAUNCH_TIMED(launch_herk_plain<R>(ctx->v.p, counts + t, nsrc, Np,
                                           static_cast<R*>(ctx->partial.p), st),
                      st);
      HV_LAUNCH(1, launch_reduce<R>(static_cast<R*>(ctx->partial.p), 0, counts + t, 1, 1, 0, 1,
                                    kPlainChunk, Np, nant, o, st));
    }
  }
  return HV_OK;
}

int dispatch_device(hv_context* ctx, int precision, int method, const void* antpos, int nant,
                    const double* freqs, int nfreq, const void* eq2tops, int ntimes,
                    const void* crd_eq, const void* I_sky, int nsrc, const void* bm, int P,
                    void* out, cudaStream_t st) {
  if (precision == 1)
    return run_device<float>(ctx, method, (const float*)antpos, nant, freqs, nfreq,
                             (const float*)eq2tops, ntimes, (const float*)crd_eq,
                             (const float*)I_sky, nsrc, (const float*)bm, P, out, st);
  return run_device<double>(ctx, method, (const double*)antpos, nant, freqs, nfreq,
                            (const double*)eq2tops, ntimes, (const double*)crd_eq,
                            (const double*)I_sky, nsrc, (const double*)bm, P, out, st);
}

// Reads (and clears) the device error flag in stream order on the context's
// stream: a copy on the legacy stream would wait on unrelated work.
int check_err_flag(hv_context* ctx) {
  int flag = 0;
  HV_CK(cudaMemcpyAsync(&flag, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  HV_CK(cudaStreamSynchronize(ctx->stream));
  if (flag != 0) {
    HV_CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
    if (flag == 2)
      return fail(ctx, HV_ERR_ARG,
                  "antenna positions x frequency exceed the FP32 phase range of the tensor-core "
                  "method (|U| >= 4e6 cycles); results of the last call are invalid, use the "
                  "plain method");
    if (flag == 3)
      return fail(ctx, HV_ERR_UNSUPPORTED,
                  "the fused kernel's dynamic shared memory is not 1024-byte aligned on this "
                  "device; results of the last call are invalid, use the plain method");
    return fail(ctx, HV_ERR_TIMEOUT,
                "a device-side wait gave up (code %d); results of the last call are invalid", flag);
  }
  return HV_OK;
}

}  // namespace

cudaStream_t hv_context_stream(hv_context* ctx) { return ctx->stream; }
void hv_context_set_error(hv_context* ctx, const char* msg) { ctx->err = msg; }
void hv_context_add_launches(hv_context* ctx, uint64_t n) { ctx->launches += n; }
int hv_context_num_sms(hv_context* ctx) { return ctx->num_sms; }

void* hv_context_host_take(hv_context* ctx, size_t bytes, size_t* cap) {
  // the smallest pooled block that fits, else a new one
  size_t best = ctx->host_pool.size();
  for (size_t i = 0; i < ctx->host_pool.size(); ++i)
    if (ctx->host_pool[i].second >= bytes &&
        (best == ctx->host_pool.size() || ctx->host_pool[i].second < ctx->host_pool[best].second))
      best = i;
  if (best < ctx->host_pool.size()) {
    void* p = ctx->host_pool[best].first;
    *cap = ctx->host_pool[best].second;
    ctx->host_pool.erase(ctx->host_pool.begin() + (long)best);
    return p;
  }
  const size_t want = std::max<size_t>(4096, bytes + bytes / 4);
  void* p = nullptr;
  if (cudaHostAlloc(&p, want, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  *cap = want;
  return p;
}

void hv_context_host_give(hv_context* ctx, void* p, size_t cap) {
  if (p) ctx->host_pool.emplace_back(p, cap);
}

void hv_context_record_kernel(hv_context* ctx, cudaEvent_t e0, cudaEvent_t e1) {
  ctx->prof_events.emplace_back(e0, e1);
}

bool hv_context_profiling(hv_context* ctx) { return ctx->profiling; }
uint64_t hv_context_wait_ns(hv_context* ctx) { return ctx->wait_ns; }
hv::TcShare* hv_context_share(hv_context* ctx) { return &ctx->share; }
int hv_context_stall(hv_context* ctx) { return ctx->stall; }

extern "C" {

int hv_version(void) { return 10000; }

int hv_create(hv_context** out, int device, size_t hbm_budget_bytes) {
  if (!out) return HV_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return HV_ERR_UNSUPPORTED;
  }
  if (device < 0 || device >= ndev) return HV_ERR_ARG;
  hv_context* ctx = new hv_context();
  ctx->device = device;
  ctx->budget = hbm_budget_bytes;
  int r = HV_OK;
  do {
    if (cudaSetDevice(device) != cudaSuccess) { r = HV_ERR_CUDA; break; }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) { r = HV_ERR_CUDA; break; }
    ctx->num_sms = prop.multiProcessorCount;
    ctx->cc_major = prop.major;
    ctx->cc_minor = prop.minor;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) { r = HV_ERR_CUDA; break; }
    // device error flag (int) and the item-claim counter of the fused
    // launches (8 bytes, at offset 8)
    if (cudaMalloc(&ctx->d_err, 16) != cudaSuccess) { r = HV_ERR_OOM; break; }
    if (cudaMemset(ctx->d_err, 0, 16) != cudaSuccess) { r = HV_ERR_CUDA; break; }
    ctx->d_claim = reinterpret_cast<unsigned long long*>(ctx->d_err + 2);
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess ||
        cudaStreamCreateWithPriority(&ctx->share.hi, cudaStreamNonBlocking, greatest) != cudaSuccess ||
        cudaStreamCreateWithPriority(&ctx->share.lo, cudaStreamNonBlocking, least) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->share.fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->share.join_hi, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->share.join_lo, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->joined, cudaEventDisableTiming) != cudaSuccess) {
      r = HV_ERR_CUDA;
      break;
    }
    // keep freed stream-ordered memory in the pool for reuse
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
      uint64_t keep = ~0ull;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  } while (0);
  if (r != HV_OK) {
    cudaGetLastError();
    hv_destroy(ctx);
    return r;
  }
  *out = ctx;
  return HV_OK;
}

int hv_destroy(hv_context* ctx) {
  if (!ctx) return HV_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  DevBuf* bufs[] = {&ctx->in_antpos, &ctx->in_eq2tops, &ctx->in_crd, &ctx->in_I, &ctx->in_bm,
                    &ctx->out_vis, &ctx->freqs, &ctx->beamT, &ctx->ucoef, &ctx->rec,
                    &ctx->counts, &ctx->blkcounts, &ctx->v, &ctx->partial, &ctx->tcgroups,
                    &ctx->umax, &ctx->sortkv, &ctx->crd_sorted, &ctx->I_sorted, &ctx->tctable,
                    &ctx->pixmax, &ctx->sbound};
  for (DevBuf* b : bufs) release(ctx, *b);
  if (ctx->tctable_h.p) cudaFreeHost(ctx->tctable_h.p);
  for (auto& hp : ctx->host_pool) cudaFreeHost(hp.first);
  for (auto& ev : ctx->prof_events) {
    cudaEventDestroy(ev.first);
    cudaEventDestroy(ev.second);
  }
  if (ctx->share.hi) cudaStreamSynchronize(ctx->share.hi);
  if (ctx->share.lo) cudaStreamSynchronize(ctx->share.lo);
  if (ctx->d_err) cudaFree(ctx->d_err);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->share.hi) cudaStreamDestroy(ctx->share.hi);
  if (ctx->share.lo) cudaStreamDestroy(ctx->share.lo);
  for (cudaEvent_t ev : {ctx->share.fork, ctx->share.join_hi, ctx->share.join_lo, ctx->joined})
    if (ev) cudaEventDestroy(ev);
  delete ctx;
  return HV_OK;
}

const char* hv_last_error(const hv_context* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

uint64_t hv_launch_count(const hv_context* ctx) { return ctx ? ctx->launches : 0; }

int hv_sync(hv_context* ctx) {
  if (!ctx) return HV_ERR_ARG;
  HV_CK(cudaSetDevice(ctx->device));
  HV_CK(cudaStreamSynchronize(ctx->stream));
  return check_err_flag(ctx);
}

int hv_vis_multifreq_device(hv_context* ctx, int precision, int method, const void* d_antpos,
                            int nant, const double* freqs, int nfreq, const void* d_eq2tops,
                            int ntimes, const void* d_crd_eq, const void* d_I_sky, int nsrc,
                            const void* d_bm_cubes, int beam_px, void* d_vis_out, void* stream) {
  if (!ctx) return HV_ERR_ARG;
  int r = check_shapes(ctx, precision, method, nant, nfreq, ntimes, nsrc, beam_px);
  if (r != HV_OK) return r;
  if (!freqs || !d_antpos || !d_eq2tops || !d_bm_cubes || !d_vis_out ||
      (nsrc > 0 && (!d_crd_eq || !d_I_sky)))
    return fail(ctx, HV_ERR_ARG, "null array argument");
  HV_CK(cudaSetDevice(ctx->device));
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  r = dispatch_device(ctx, precision, method, d_antpos, nant, freqs, nfreq, d_eq2tops, ntimes,
                      d_crd_eq, d_I_sky, nsrc, d_bm_cubes, beam_px, d_vis_out, st);
  if (r != HV_OK || st == ctx->stream) return r;
  // the context's stream follows the call's work (not while the caller's
  // stream is being captured: that would pull the context's stream into the
  // capture), so that hv_sync waits for it and reads its error flag after it
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  HV_CK(cudaStreamIsCapturing(st, &cap));
  if (cap == cudaStreamCaptureStatusNone) {
    HV_CK(cudaEventRecord(ctx->joined, st));
    HV_CK(cudaStreamWaitEvent(ctx->stream, ctx->joined, 0));
  }
  return HV_OK;
}

int hv_vis_multifreq(hv_context* ctx, int precision, int method, const void* antpos, int nant,
                     const double* freqs, int nfreq, const void* eq2tops, int ntimes,
                     const void* crd_eq, const void* I_sky, int nsrc, const void* bm_cubes,
                     int beam_px, void* vis_out) {
  if (!ctx) return HV_ERR_ARG;
  int r = check_shapes(ctx, precision, method, nant, nfreq, ntimes, nsrc, beam_px);
  if (r != HV_OK) return r;
  if (!freqs || !antpos || !eq2tops || !bm_cubes || !vis_out ||
      (nsrc > 0 && (!crd_eq || !I_sky)))
    return fail(ctx, HV_ERR_ARG, "null array argument");
  HV_CK(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  const size_t rs = precision == 1 ? 4 : 8;
  const size_t b_antpos = rs * nant * 3, b_e2t = rs * (size_t)ntimes * 9,
               b_crd = rs * 3 * (size_t)nsrc, b_I = rs * (size_t)nsrc,
               b_bm = rs * (size_t)nfreq * nant * beam_px * beam_px,
               b_out = 2 * rs * (size_t)nfreq * ntimes * nant * nant;
  HV_ENSURE(ctx->in_antpos, b_antpos);
  HV_ENSURE(ctx->in_eq2tops, b_e2t);
  HV_ENSURE(ctx->in_crd, b_crd);
  HV_ENSURE(ctx->in_I, b_I);
  HV_ENSURE(ctx->in_bm, b_bm);
  HV_ENSURE(ctx->out_vis, b_out);
  HV_CK(cudaMemcpyAsync(ctx->in_antpos.p, antpos, b_antpos, cudaMemcpyHostToDevice, st));
  if (b_e2t) HV_CK(cudaMemcpyAsync(ctx->in_eq2tops.p, eq2tops, b_e2t, cudaMemcpyHostToDevice, st));
  if (b_crd) HV_CK(cudaMemcpyAsync(ctx->in_crd.p, crd_eq, b_crd, cudaMemcpyHostToDevice, st));
  if (b_I) HV_CK(cudaMemcpyAsync(ctx->in_I.p, I_sky, b_I, cudaMemcpyHostToDevice, st));
  HV_CK(cudaMemcpyAsync(ctx->in_bm.p, bm_cubes, b_bm, cudaMemcpyHostToDevice, st));
  r = dispatch_device(ctx, precision, method, ctx->in_antpos.p, nant, freqs, nfreq,
                      ctx->in_eq2tops.p, ntimes, ctx->in_crd.p, ctx->in_I.p, nsrc,
                      ctx->in_bm.p, beam_px, ctx->out_vis.p, st);
  if (r != HV_OK) {
    cudaStreamSynchronize(st);
    return r;
  }
  if (b_out) HV_CK(cudaMemcpyAsync(vis_out, ctx->out_vis.p, b_out, cudaMemcpyDeviceToHost, st));
  HV_CK(cudaStreamSynchronize(st));
  return check_err_flag(ctx);
}

int hv_vis_gpu(hv_context* ctx, int precision, int method, const void* antpos, int nant,
               double freq, const void* eq2tops, int ntimes, const void* crd_eq,
               const void* I_sky, int nsrc, const void* bm_cube, int beam_px, void* vis_out) {
  return hv_vis_multifreq(ctx, precision, method, antpos, nant, &freq, 1, eq2tops, ntimes,
                          crd_eq, I_sky, nsrc, bm_cube, beam_px, vis_out);
}

int hv_set_profiling(hv_context* ctx, int enable) {
  if (!ctx) return HV_ERR_ARG;
  ctx->profiling = enable != 0;
  return HV_OK;
}

int hv_set_tuning(hv_context* ctx, int param, int value) {
  if (!ctx) return HV_ERR_ARG;
  switch (param) {
    case HV_TUNE_STAGES:
      if (value != 0 && (value < 2 || value > 8))
        return fail(ctx, HV_ERR_ARG, "stages must be 0 or in [2, 8] (got %d)", value);
      ctx->tune.stages = value;
      return HV_OK;
    default:
      return fail(ctx, HV_ERR_ARG, "unknown tuning parameter %d", param);
  }
}

int hv_set_wait_limit(hv_context* ctx, uint64_t wait_ns, int stall) {
  if (!ctx) return HV_ERR_ARG;
  ctx->wait_ns = wait_ns;
  ctx->stall = stall != 0;
  return HV_OK;
}

int hv_profile_read(hv_context* ctx, double* ms, uint64_t* launches) {
  if (!ctx || !ms || !launches) return HV_ERR_ARG;
  HV_CK(cudaSetDevice(ctx->device));
  double total = 0.0;
  for (auto& ev : ctx->prof_events) {
    HV_CK(cudaEventSynchronize(ev.second));
    float t = 0.f;
    HV_CK(cudaEventElapsedTime(&t, ev.first, ev.second));
    total += t;
  }
  *ms = total;
  *launches = ctx->prof_events.size();
  for (auto& ev : ctx->prof_events) {
    cudaEventDestroy(ev.first);
    cudaEventDestroy(ev.second);
  }
  ctx->prof_events.clear();
  return HV_OK;
}

int hv_device_alloc(hv_context* ctx, size_t bytes, void** ptr) {
  if (!ctx || !ptr) return HV_ERR_ARG;
  HV_CK(cudaSetDevice(ctx->device));
  cudaError_t e = cudaMallocAsync(ptr, bytes ? bytes : 1, ctx->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, HV_ERR_OOM, "cudaMallocAsync(%zu) failed: %s", bytes, cudaGetErrorString(e));
  }
  return HV_OK;
}

int hv_device_free(hv_context* ctx, void* ptr) {
  if (!ctx) return HV_ERR_ARG;
  if (ptr) HV_CK(cudaFreeAsync(ptr, ctx->stream));
  return HV_OK;
}

int hv_memcpy_async(hv_context* ctx, void* dst, const void* src, size_t bytes, int kind) {
  if (!ctx || (bytes && (!dst || !src)) || kind < 1 || kind > 3) return HV_ERR_ARG;
  if (!bytes) return HV_OK;
  const cudaMemcpyKind k = kind == 1 ? cudaMemcpyHostToDevice
                           : kind == 2 ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  HV_CK(cudaMemcpyAsync(dst, src, bytes, k, ctx->stream));
  return HV_OK;
}

int hv_stream_query(hv_context* ctx) {
  if (!ctx) return -HV_ERR_ARG;
  const cudaError_t e = cudaStreamQuery(ctx->stream);
  if (e == cudaSuccess) return 0;
  if (e == cudaErrorNotReady) return 1;
  ctx->err = cudaGetErrorString(e);
  return -HV_ERR_CUDA;
}

int hv_host_alloc(hv_context* ctx, size_t bytes, void** ptr) {
  if (!ctx || !ptr) return HV_ERR_ARG;
  HV_CK(cudaSetDevice(ctx->device));
  HV_CK(cudaHostAlloc(ptr, bytes ? bytes : 1, cudaHostAllocDefault));
  return HV_OK;
}

int hv_host_free(hv_context* ctx, void* ptr) {
  if (!ctx) return HV_ERR_ARG;
  if (ptr) HV_CK(cudaFreeHost(ptr));
  return HV_OK;
}

}  // extern "C"
