// hv_batch.cu -- many independent simulations in one go (batched form).
//
// The reference simulates one (antenna layout, sky, beam, frequency) per call
// (hera_gpu/vis.py:144); a batch of uneven simulations would be a loop of
// calls, each too small to fill a GB300.  Here a batch is planned once:
//   * one device arena holds every simulation's working memory (beams in
//     [pixel][antenna] layout, phase coefficients, sorted catalogue, source
//     records, split-K partial sums);
//   * the preparation kernels run per simulation (they are small);
//   * the fused tensor-core kernel runs ONE persistent launch per cluster
//     class (simulations with the same 128-antenna block count share a
//     cluster layout), over the items of all of that class's simulations;
//   * a reduction per simulation writes its (nfreq, ntimes, nant, nant)
//     output.
// The whole sequence can be captured once into a CUDA graph and replayed
// (hv_batch_launch); the split-K depth of each class can be picked by timing
// candidates on the batch itself (hv_batch_create with HV_BATCH_AUTOTUNE).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "heravis.h"
#include "hv_internal.cuh"
#include "hv_kernels.h"

namespace {

size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

struct SimPlan {
  hv_sim in;
  int Np, ngroups, max_slots, nchunk, chunk, rec_stride;
  long long rec_row0;
  size_t o_freqs, o_beam, o_U, o_umax, o_counts, o_blk, o_kv, o_crd, o_I, o_partial, o_groups;
  size_t h_freqs;    // offset of the frequencies in the pinned host block
  size_t h_groups;   // offset of its group table in the pinned host block
  int cls;           // index of its cluster class
};

}  // namespace

struct hv_batch {
  hv_context* ctx = nullptr;
  int device = 0;
  int num_sms = 0;
  std::vector<SimPlan> sims;
  std::vector<std::vector<int>> classes;   // simulation indices per class
  std::vector<int> class_nchunk_div;       // split-K divisor per class
  void* arena = nullptr;                   // device
  size_t arena_bytes = 0;
  void* rec = nullptr;                     // device records of every simulation
  long long rec_rows = 0;
  void* table = nullptr;                   // device simulation tables, per class
  void* host = nullptr;                    // pinned: frequencies, group tables, sim tables
  size_t host_cap = 0;                     // its size (a block of the context's pool)
  size_t host_bytes = 0, h_table = 0, h_groups = 0;
  int* d_err = nullptr;                    // error flag (int) and, at offset 8, the
  unsigned long long* d_claim = nullptr;   // item-claim counter of its fused launches
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::string err;
  uint64_t launches_per_run = 0;
};

namespace {

int bfail(hv_batch* b, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (b) b->err = buf;
  return code;
}

#define HB_CK(call)                                                                       \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return bfail(b, HV_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));       \
  } while (0)

int rec_stride_of(int nsrc) { return ((std::max(nsrc, 1) + 31) / 32) * 32; }

// Split-K of a batch: a slice's sources are cut into chunks of at most
// kBatchChunk (divided further by the class's autotuned divisor), so that
// one item of the persistent launch stays within a few milliseconds and a
// large simulation spreads over every SM.  The cut depends on the
// simulation alone: its result does not depend on the batch it runs in.
constexpr int kBatchChunk = 65536;

void chunking(int nsrc, int div, int* chunk, int* nchunk) {
  const int S = std::max(nsrc, 1);
  const int parts = hv::ceil_div(S, kBatchChunk) * std::max(div, 1);
  *chunk = std::max(32, hv::ceil_div(hv::ceil_div(S, parts), 32) * 32);
  *nchunk = hv::ceil_div(S, *chunk);
}

// Lay out every simulation in the arena (split-K depth from the class divisor).
void layout(hv_batch* b) {
  size_t off = 0, hoff = 0;
  long long rows = 0;
  std::map<int, std::pair<size_t, size_t>> groups_at;  // nant -> (device, host) offsets
  for (auto& s : b->sims) {
    const hv_sim& in = s.in;
    const int T = in.ntimes, F = in.nfreq, S = in.nsrc, P = in.beam_px;
    s.Np = hv::ceil_div(in.nant, hv::kAntPad) * hv::kAntPad;
    const int div = b->class_nchunk_div.empty() ? 1 : b->class_nchunk_div[s.cls];
    chunking(S, div, &s.chunk, &s.nchunk);
    s.rec_stride = rec_stride_of(S);
    s.rec_row0 = rows;
    rows += (long long)T * s.rec_stride;
    s.o_freqs = off; off += up256(sizeof(double) * F);
    s.o_beam = off; off += up256(sizeof(float) * (size_t)F * P * P * s.Np);
    s.o_U = off; off += up256(sizeof(hv::Ucoef32) * (size_t)T * F * s.Np);
    s.o_umax = off; off += up256(sizeof(float) * (size_t)T * F);
    s.o_counts = off; off += up256(sizeof(int) * (size_t)std::max(T, 1));
    s.o_blk = off; off += up256(sizeof(int) * (size_t)T * hv::prep_blocks(S));
    s.o_kv = off; off += up256(sizeof(unsigned long long) * (size_t)hv::sort_pad(std::max(S, 1)));
    s.o_crd = off; off += up256(sizeof(float) * 3 * (size_t)std::max(S, 1));
    s.o_I = off; off += up256(sizeof(float) * (size_t)std::max(S, 1));
    s.o_partial = off;
    off += up256(sizeof(float) * (size_t)T * F * s.nchunk * 2 * s.Np * s.Np);
    auto it = groups_at.find(in.nant);
    if (it == groups_at.end()) {
      const size_t gb = hv::tc_group_table_bytes(in.nant);
      groups_at[in.nant] = {off, hoff};
      s.o_groups = off;
      s.h_groups = hoff;
      off += up256(gb);
      hoff += up256(gb);
    } else {
      s.o_groups = it->second.first;
      s.h_groups = it->second.second;
    }
    s.h_freqs = hoff;
    hoff += up256(sizeof(double) * F);
  }
  b->arena_bytes = off;
  b->rec_rows = rows;
  b->h_groups = 0;
  b->h_table = hoff;
  // one simulation table per class (an empty class still takes one entry)
  b->host_bytes = hoff + up256(hv::tc_sim_table_bytes((int)(b->sims.size() + b->classes.size())));
}

// Device memory of the batch comes from the stream-ordered pool of the
// context's stream: creating and destroying batches does not stall work on
// other streams.
void release(hv_batch* b) {
  cudaStream_t st = hv_context_stream(b->ctx);
  if (b->arena) cudaFreeAsync(b->arena, st);
  if (b->rec) cudaFreeAsync(b->rec, st);
  if (b->table) cudaFreeAsync(b->table, st);
  b->arena = b->rec = b->table = nullptr;
}

int allocate(hv_batch* b) {
  cudaStream_t st = hv_context_stream(b->ctx);
  release(b);
  if (b->host && b->host_cap < b->host_bytes) {
    cudaStreamSynchronize(st);  // the host block may still feed queued copies
    hv_context_host_give(b->ctx, b->host, b->host_cap);
    b->host = nullptr;
  }
  HB_CK(cudaMallocAsync(&b->arena, std::max<size_t>(b->arena_bytes, 256), st));
  HB_CK(cudaMallocAsync(&b->rec, sizeof(hv::SrcRec32) * (size_t)std::max<long long>(b->rec_rows, 1), st));
  HB_CK(cudaMallocAsync(&b->table, hv::tc_sim_table_bytes((int)(b->sims.size() + b->classes.size())), st));
  if (!b->host) {
    b->host = hv_context_host_take(b->ctx, std::max<size_t>(b->host_bytes, 256), &b->host_cap);
    if (!b->host) return bfail(b, HV_ERR_OOM, "page-locked host block of %zu bytes", b->host_bytes);
  }
  // constant host data: frequencies and group tables
  char* h = static_cast<char*>(b->host);
  for (auto& s : b->sims) {
    hv::tc_fill_group_table(s.in.nant, h + s.h_groups);
    std::memcpy(h + s.h_freqs, s.in.freqs, sizeof(double) * s.in.nfreq);
  }
  return HV_OK;
}

// All work of the batch on stream st (no allocation, no synchronisation:
// safe under stream capture).  timed_class >= 0: only the fused launch of
// that class (for the autotuner).
int enqueue(hv_batch* b, cudaStream_t st, int timed_class = -1) {
  using namespace hv;
  char* A = static_cast<char*>(b->arena);
  char* H = static_cast<char*>(b->host);
  uint64_t nl = 0;
  std::map<int, bool> groups_copied;
  if (timed_class < 0) {
    for (auto& s : b->sims) {
      const hv_sim& in = s.in;
      const int T = in.ntimes, F = in.nfreq, S = in.nsrc, P = in.beam_px;
      if (!groups_copied[in.nant]) {
        groups_copied[in.nant] = true;
        HB_CK(cudaMemcpyAsync(A + s.o_groups, H + s.h_groups, tc_group_table_bytes(in.nant),
                              cudaMemcpyHostToDevice, st));
      }
      if (T == 0) continue;
      HB_CK(cudaMemcpyAsync(A + s.o_freqs, H + s.h_freqs, sizeof(double) * F,
                            cudaMemcpyHostToDevice, st));
      float* beamT = reinterpret_cast<float*>(A + s.o_beam);
      HB_CK(launch_beam_transpose<float>(in.bm_cubes, F, in.nant, P, s.Np, beamT, st));
      HB_CK(launch_ucoef<float>(in.antpos, in.nant, s.Np, in.eq2tops, 0, T,
                                reinterpret_cast<const double*>(A + s.o_freqs), F, A + s.o_U, st));
      HB_CK(launch_ubound(A + s.o_U, T * F, s.Np, reinterpret_cast<float*>(A + s.o_umax), st));
      nl += 3;
      const float* crd = in.crd_eq;
      const float* I = in.I_sky;
      if (S > 0) {
        int k = 0;
        HB_CK(launch_sort_sources(in.crd_eq, in.I_sky, S, A + s.o_kv,
                                  reinterpret_cast<float*>(A + s.o_crd),
                                  reinterpret_cast<float*>(A + s.o_I), &k, st));
        nl += k;
        crd = reinterpret_cast<const float*>(A + s.o_crd);
        I = reinterpret_cast<const float*>(A + s.o_I);
      }
      SrcRec32* rec = static_cast<SrcRec32*>(b->rec) + s.rec_row0;
      HB_CK(launch_prep_strided<float>(crd, I, S, in.eq2tops, 0, T, P,
                                       reinterpret_cast<int*>(A + s.o_blk), rec,
                                       (size_t)s.rec_stride,
                                       reinterpret_cast<int*>(A + s.o_counts), st));
      HB_CK(launch_tc_relative(rec, (size_t)s.rec_stride, reinterpret_cast<int*>(A + s.o_counts),
                               T, S, st));
      nl += 3;
    }
  }
  // one persistent fused launch per class; its CTAs claim the items in
  // table order, so the simulations with the largest items go first and the
  // small ones fill the tail
  size_t toff = 0;
  for (size_t c = 0; c < b->classes.size(); ++c) {
    std::vector<int> order = b->classes[c];
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
      const SimPlan &sx = b->sims[x], &sy = b->sims[y];
      return std::min(sx.chunk, sx.in.nsrc) > std::min(sy.chunk, sy.in.nsrc);
    });
    std::vector<TcSimDesc> d;
    for (int i : order) {
      const SimPlan& s = b->sims[i];
      if (s.in.ntimes == 0 || s.in.nsrc == 0) continue;
      TcSimDesc x{};
      x.counts = reinterpret_cast<const int*>(A + s.o_counts);
      x.U = A + s.o_U;
      x.beamT = reinterpret_cast<const float*>(A + s.o_beam);
      x.umax = reinterpret_cast<const float*>(A + s.o_umax);
      x.partial = reinterpret_cast<float*>(A + s.o_partial);
      x.groups = A + s.o_groups;
      x.ngroups = s.ngroups;
      x.max_slots = s.max_slots;
      x.rec_row0 = s.rec_row0;
      x.rec_stride = s.rec_stride;
      x.nt = s.in.ntimes;
      x.nf = s.in.nfreq;
      x.Np = s.Np;
      x.nant = s.in.nant;
      x.P = s.in.beam_px;
      x.nsrc = s.in.nsrc;
      x.chunk = s.chunk;
      d.push_back(x);
    }
    if (!d.empty() && (timed_class < 0 || timed_class == (int)c)) {
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      const bool prof = timed_class < 0 && hv_context_profiling(b->ctx) &&
                        cudaStreamIsCapturing(st, &cs) == cudaSuccess &&
                        cs == cudaStreamCaptureStatusNone;
      if (prof) {
        HB_CK(cudaEventCreate(&e0));
        HB_CK(cudaEventCreate(&e1));
        HB_CK(cudaEventRecord(e0, st));
      }
      // a class of one simulation in cluster mode shares its launch with the
      // SMs no cluster fits on (not while timing split-K candidates)
      TcShare* share = d.size() == 1 && timed_class < 0 ? hv_context_share(b->ctx) : nullptr;
      HB_CK(launch_tc_batch(d.data(), (int)d.size(), b->rec, b->rec_rows,
                            static_cast<char*>(b->table) + toff, H + b->h_table + toff, b->d_err,
                            b->d_claim, b->num_sms, st, hv_context_wait_ns(b->ctx),
                            hv_context_stall(b->ctx), share));
      if (share && share->launched > 1) nl += share->launched - 1;
      if (prof) {
        HB_CK(cudaEventRecord(e1, st));
        hv_context_record_kernel(b->ctx, e0, e1);
      }
      ++nl;
    }
    toff += tc_sim_table_bytes((int)d.size());
  }
  if (timed_class < 0) {
    for (auto& s : b->sims) {
      const hv_sim& in = s.in;
      if (in.ntimes == 0) continue;
      const size_t slice = (size_t)s.nchunk * 2 * s.Np * s.Np;
      HB_CK(launch_reduce<float>(reinterpret_cast<float*>(A + s.o_partial), slice,
                                 reinterpret_cast<const int*>(A + s.o_counts), in.ntimes,
                                 in.nfreq, 0, in.ntimes, s.chunk, s.Np, in.nant, in.vis_out, st));
      ++nl;
    }
    b->launches_per_run = nl;
  }
  return HV_OK;
}

int check_sim(hv_batch* b, const hv_sim& s, int i) {
  if (s.nant < 1 || s.nant > 65536 || s.ntimes < 0 || s.nsrc < 0 || s.nfreq < 1 ||
      s.beam_px < 1 || s.beam_px > 4096 || (long long)s.ntimes * s.nfreq > 0x7fffffffLL)
    return bfail(b, HV_ERR_ARG, "simulation %d: bad sizes (nant %d ntimes %d nsrc %d nfreq %d P %d)",
                 i, s.nant, s.ntimes, s.nsrc, s.nfreq, s.beam_px);
  if (!s.antpos || !s.eq2tops || !s.bm_cubes || !s.freqs || !s.vis_out ||
      (s.nsrc > 0 && (!s.crd_eq || !s.I_sky)))
    return bfail(b, HV_ERR_ARG, "simulation %d: null array", i);
  return HV_OK;
}

}  // namespace

extern "C" {

int hv_batch_create(hv_context* ctx, const hv_sim* sims, int nsims, unsigned flags,
                    hv_batch** out) {
  if (!ctx || !out || nsims < 1 || !sims) return HV_ERR_ARG;
  *out = nullptr;
  hv_batch* b = new hv_batch();
  b->ctx = ctx;
  int r = HV_OK;
  do {
    if (cudaGetDevice(&b->device) != cudaSuccess) { r = HV_ERR_CUDA; break; }
    b->num_sms = hv_context_num_sms(ctx);
    if (cudaMallocAsync(reinterpret_cast<void**>(&b->d_err), 16, hv_context_stream(ctx)) !=
        cudaSuccess) { r = HV_ERR_OOM; break; }
    cudaMemsetAsync(b->d_err, 0, 16, hv_context_stream(ctx));
    b->d_claim = reinterpret_cast<unsigned long long*>(b->d_err + 2);
    std::map<int, int> class_of;  // cluster size (0 = no cluster) -> class
    for (int i = 0; i < nsims; ++i) {
      r = check_sim(b, sims[i], i);
      if (r != HV_OK) break;
      SimPlan s{};
      s.in = sims[i];
      s.ngroups = hv::tc_num_groups(sims[i].nant);
      s.max_slots = hv::tc_max_slots(sims[i].nant);
      // cluster classes by cluster size; the others by generator team size
      const int key = (s.ngroups > 1 && s.ngroups <= 8) ? s.ngroups
                                                        : 100 + hv::tc_team_warps(sims[i].nant);
      auto it = class_of.find(key);
      if (it == class_of.end()) {
        class_of[key] = (int)b->classes.size();
        b->classes.push_back({});
      }
      s.cls = class_of[key];
      b->classes[s.cls].push_back(i);
      b->sims.push_back(s);
    }
    if (r != HV_OK) break;
    b->class_nchunk_div.assign(b->classes.size(), 1);
    layout(b);
    r = allocate(b);
    if (r != HV_OK) break;
    cudaStream_t st = hv_context_stream(ctx);
    if (hv::tc_configure() != cudaSuccess) { r = HV_ERR_CUDA; break; }
    if (flags & HV_BATCH_AUTOTUNE) {
      // split-K depth per class: time the fused launch with 1, 2 and 4
      // chunks per slice on this batch and keep the fastest
      r = enqueue(b, st);
      if (r != HV_OK) break;
      std::vector<int> best(b->classes.size(), 1);
      for (size_t c = 0; c < b->classes.size() && r == HV_OK; ++c) {
        float best_ms = 1e30f;
        for (int div : {1, 2, 4}) {
          b->class_nchunk_div[c] = div;
          layout(b);
          r = allocate(b);
          if (r != HV_OK) break;
          r = enqueue(b, st);  // preparation for this layout
          if (r != HV_OK) break;
          cudaEvent_t e0, e1;
          cudaEventCreate(&e0);
          cudaEventCreate(&e1);
          cudaEventRecord(e0, st);
          r = enqueue(b, st, (int)c);
          cudaEventRecord(e1, st);
          cudaEventSynchronize(e1);
          float ms = 0.f;
          cudaEventElapsedTime(&ms, e0, e1);
          cudaEventDestroy(e0);
          cudaEventDestroy(e1);
          if (ms < best_ms) {
            best_ms = ms;
            best[c] = div;
          }
        }
        b->class_nchunk_div[c] = best[c];
      }
      if (r != HV_OK) break;
      layout(b);
      r = allocate(b);
      if (r != HV_OK) break;
    }
    if (flags & HV_BATCH_GRAPH) {
      if (cudaStreamSynchronize(st) != cudaSuccess) { r = HV_ERR_CUDA; break; }
      if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        r = HV_ERR_CUDA;
        break;
      }
      r = enqueue(b, st);
      cudaGraph_t g = nullptr;
      const cudaError_t ec = cudaStreamEndCapture(st, &g);
      if (r != HV_OK) break;
      if (ec != cudaSuccess) { r = bfail(b, HV_ERR_CUDA, "stream capture failed: %s", cudaGetErrorString(ec)); break; }
      b->graph = g;
      if (cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) { r = HV_ERR_CUDA; break; }
    }
    // allocations and constant copies done before the batch may run elsewhere
    if (cudaStreamSynchronize(st) != cudaSuccess) { r = HV_ERR_CUDA; break; }
  } while (0);
  if (r != HV_OK) {
    if (ctx) hv_context_set_error(ctx, b->err.empty() ? "hv_batch_create failed" : b->err.c_str());
    hv_batch_destroy(b);
    return r;
  }
  *out = b;
  return HV_OK;
}

int hv_batch_launch(hv_batch* b, void* stream) {
  if (!b) return HV_ERR_ARG;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : hv_context_stream(b->ctx);
  if (b->exec) {
    if (cudaGraphLaunch(b->exec, st) != cudaSuccess) return HV_ERR_CUDA;
    hv_context_add_launches(b->ctx, b->launches_per_run);
    return HV_OK;
  }
  const int r = enqueue(b, st);
  if (r != HV_OK) {
    hv_context_set_error(b->ctx, b->err.c_str());
    return r;
  }
  hv_context_add_launches(b->ctx, b->launches_per_run);
  return HV_OK;
}

int hv_batch_sync(hv_batch* b) {
  if (!b) return HV_ERR_ARG;
  // the error flag is read in stream order on the batch's stream (a copy on
  // the legacy stream would wait on the other streams' work)
  cudaStream_t st = hv_context_stream(b->ctx);
  int flag = 0;
  if (cudaMemcpyAsync(&flag, b->d_err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return HV_ERR_CUDA;
  if (flag) {
    cudaMemsetAsync(b->d_err, 0, sizeof(int), st);
    return flag == 2 ? HV_ERR_ARG : flag == 3 ? HV_ERR_UNSUPPORTED : HV_ERR_TIMEOUT;
  }
  return HV_OK;
}

uint64_t hv_batch_launches(const hv_batch* b) { return b ? b->launches_per_run : 0; }

int hv_batch_destroy(hv_batch* b) {
  if (!b) return HV_OK;
  // runs of the batch are ordered on the context's stream (or were waited
  // for by the caller): release after them
  if (b->ctx) {
    cudaStreamSynchronize(hv_context_stream(b->ctx));
    release(b);
  }
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->host) hv_context_host_give(b->ctx, b->host, b->host_cap);
  if (b->d_err) cudaFreeAsync(b->d_err, hv_context_stream(b->ctx));
  delete b;
  return HV_OK;
}

int hv_vis_batch(hv_context* ctx, const hv_sim* sims, int nsims, void* stream) {
  hv_batch* b = nullptr;
  int r = hv_batch_create(ctx, sims, nsims, 0, &b);
  if (r != HV_OK) return r;
  r = hv_batch_launch(b, stream);
  if (r == HV_OK) r = hv_batch_sync(b);
  if (r != HV_OK && ctx) hv_context_set_error(ctx, b->err.empty() ? "batch failed" : b->err.c_str());
  hv_batch_destroy(b);
  return r;
}

}  // extern "C"
