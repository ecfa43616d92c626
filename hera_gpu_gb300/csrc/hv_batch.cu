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
  size_t o_beam, o_U, o_umax, o_counts, o_blk, o_kv, o_crd, o_I, o_partial;
  // offsets in the constant block (the same in the pinned host block and at
  // the start of the device arena)
  size_t c_freqs, c_groups;
  int cls;           // index of its cluster class
};

// Prefix tables of the table-driven batch launches, in PrepPre's order.
constexpr int kPrepTables = 9;

}  // namespace

struct hv_batch {
  hv_context* ctx = nullptr;
  int device = 0;
  int num_sms = 0;
  std::vector<SimPlan> sims;
  std::vector<std::vector<int>> classes;   // simulation indices per class
  std::vector<int> class_nchunk_div;       // split-K divisor per class
  std::vector<int> class_stages;           // operand-stage cap per class (0: as many as fit)
  void* arena = nullptr;                   // device: the constant block, then the work areas
  size_t arena_bytes = 0;
  // constant block: group tables, frequencies, the PrepSim table and the
  // prefix tables; written once per layout and copied to the arena's start
  size_t const_bytes = 0, c_prep = 0, c_pre = 0;
  hv::PrepTotals totals{};
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

// Lay out every simulation in the arena (split-K depth from the class
// divisor): the constant block first, then each simulation's work areas.
void layout(hv_batch* b) {
  const int n = (int)b->sims.size();
  // constant block: group tables (one per antenna count), frequencies,
  // PrepSim table, prefix tables
  size_t c = 0;
  std::map<int, size_t> groups_at;  // nant -> offset
  for (auto& s : b->sims) {
    auto it = groups_at.find(s.in.nant);
    if (it == groups_at.end()) {
      groups_at[s.in.nant] = c;
      s.c_groups = c;
      c += up256(hv::tc_group_table_bytes(s.in.nant));
    } else {
      s.c_groups = it->second;
    }
    s.c_freqs = c;
    c += up256(sizeof(double) * s.in.nfreq);
  }
  b->c_prep = c;
  c += up256(sizeof(hv::PrepSim) * (size_t)n);
  b->c_pre = c;
  c += up256(sizeof(long long) * (size_t)(n + 1) * kPrepTables);
  b->const_bytes = c;
  size_t off = c;
  long long rows = 0;
  for (auto& s : b->sims) {
    const hv_sim& in = s.in;
    const int T = in.ntimes, F = in.nfreq, S = in.nsrc, P = in.beam_px;
    s.Np = hv::ceil_div(in.nant, hv::kAntPad) * hv::kAntPad;
    const int div = b->class_nchunk_div.empty() ? 1 : b->class_nchunk_div[s.cls];
    chunking(S, div, &s.chunk, &s.nchunk);
    s.rec_stride = rec_stride_of(S);
    s.rec_row0 = rows;
    rows += (long long)T * s.rec_stride;
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
  }
  b->arena_bytes = off;
  b->rec_rows = rows;
  // host block: the constant block, then one fused-kernel simulation table
  // per class (an empty class still takes one entry)
  b->h_table = c;
  b->host_bytes = c + up256(hv::tc_sim_table_bytes((int)(b->sims.size() + b->classes.size())));
}

// The constant block in the host block: group tables, frequencies, the
// PrepSim table (device addresses in the arena) and the prefix tables; and
// the totals of the table-driven launches.
void fill_constants(hv_batch* b) {
  using namespace hv;
  char* H = static_cast<char*>(b->host);
  char* A = static_cast<char*>(b->arena);
  const int n = (int)b->sims.size();
  PrepSim* ps = reinterpret_cast<PrepSim*>(H + b->c_prep);
  long long* pre = reinterpret_cast<long long*>(H + b->c_pre);
  long long* pbeam = pre, *pucoef = pre + (n + 1), *pslice = pre + 2 * (n + 1),
             *pkey = pre + 3 * (n + 1), *ppair = pre + 4 * (n + 1), *ptile = pre + 5 * (n + 1),
             *pprep = pre + 6 * (n + 1), *prel = pre + 7 * (n + 1), *pred = pre + 8 * (n + 1);
  PrepTotals t{};
  for (int i = 0; i < n; ++i) {
    SimPlan& s = b->sims[i];
    const hv_sim& in = s.in;
    tc_fill_group_table(in.nant, H + s.c_groups);
    std::memcpy(H + s.c_freqs, in.freqs, sizeof(double) * in.nfreq);
    const int T = in.ntimes, F = in.nfreq, S = in.nsrc, P = in.beam_px;
    PrepSim x{};
    x.antpos = in.antpos;
    x.eq2tops = in.eq2tops;
    x.crd_eq = in.crd_eq;
    x.I_sky = in.I_sky;
    x.bm = in.bm_cubes;
    x.freqs = reinterpret_cast<const double*>(A + s.c_freqs);
    x.beamT = reinterpret_cast<float*>(A + s.o_beam);
    x.U = A + s.o_U;
    x.umax = reinterpret_cast<float*>(A + s.o_umax);
    x.counts = reinterpret_cast<int*>(A + s.o_counts);
    x.blk = reinterpret_cast<int*>(A + s.o_blk);
    x.kv = reinterpret_cast<unsigned long long*>(A + s.o_kv);
    x.crd_s = reinterpret_cast<float*>(A + s.o_crd);
    x.I_s = reinterpret_cast<float*>(A + s.o_I);
    x.rec = static_cast<SrcRec32*>(b->rec) + s.rec_row0;
    x.partial = reinterpret_cast<float*>(A + s.o_partial);
    x.out = in.vis_out;
    x.nant = in.nant;
    x.Np = s.Np;
    x.T = T;
    x.F = F;
    x.S = S;
    x.P = P;
    x.rec_stride = s.rec_stride;
    x.chunk = s.chunk;
    ps[i] = x;
    // a simulation without times has nothing to prepare or reduce
    const long long live = T > 0 ? 1 : 0;
    const int nbt = ceil_div(in.nant, 32);
    const long long key = (live && S > 0) ? sort_pad(S) : 0;
    pbeam[i] = t.beam;   t.beam += live * (long long)ceil_div((long long)P * P, 32) * (s.Np / 32) * F;
    pucoef[i] = t.ucoef; t.ucoef += (long long)T * F * s.Np;
    pslice[i] = t.slice; t.slice += (long long)T * F;
    pkey[i] = t.key;     t.key += key;
    ppair[i] = t.pair;   t.pair += key / 2;
    ptile[i] = t.tile;   t.tile += key / 2048;
    pprep[i] = t.prep;   t.prep += (long long)prep_blocks(S) * T;
    prel[i] = t.rel;     t.rel += (long long)ceil_div(s.rec_stride, 256) * T;
    pred[i] = t.red;     t.red += (long long)nbt * (nbt + 1) / 2 * T * F;
    t.max_key = std::max<long long>(t.max_key, key);
  }
  pbeam[n] = t.beam;
  pucoef[n] = t.ucoef;
  pslice[n] = t.slice;
  pkey[n] = t.key;
  ppair[n] = t.pair;
  ptile[n] = t.tile;
  pprep[n] = t.prep;
  prel[n] = t.rel;
  pred[n] = t.red;
  b->totals = t;
}

hv::PrepPre device_pre(hv_batch* b) {
  const int n = (int)b->sims.size();
  const long long* pre = reinterpret_cast<const long long*>(static_cast<char*>(b->arena) + b->c_pre);
  hv::PrepPre p{};
  p.beam = pre;
  p.ucoef = pre + (n + 1);
  p.slice = pre + 2 * (n + 1);
  p.key = pre + 3 * (n + 1);
  p.pair = pre + 4 * (n + 1);
  p.tile = pre + 5 * (n + 1);
  p.prep = pre + 6 * (n + 1);
  p.rel = pre + 7 * (n + 1);
  p.red = pre + 8 * (n + 1);
  return p;
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
  // the constant block, copied once per layout (it does not change between
  // runs; the caller synchronises before the batch runs or is captured)
  fill_constants(b);
  HB_CK(cudaMemcpyAsync(b->arena, b->host, b->const_bytes, cudaMemcpyHostToDevice, st));
  return HV_OK;
}

// All work of the batch on stream st (no allocation, no synchronisation:
// safe under stream capture).  timed_class >= 0: only the fused launch of
// that class (for the autotuner).  The preparation and the reduction of
// every simulation are table-driven launches over the whole batch.
int enqueue(hv_batch* b, cudaStream_t st, int timed_class = -1) {
  using namespace hv;
  char* A = static_cast<char*>(b->arena);
  char* H = static_cast<char*>(b->host);
  uint64_t nl = 0;
  const PrepSim* sims = reinterpret_cast<const PrepSim*>(A + b->c_prep);
  const PrepPre pre = device_pre(b);
  const int n = (int)b->sims.size();
  if (timed_class < 0) {
    int k = 0;
    HB_CK(launch_prepare_batch(sims, n, pre, b->totals, &k, st));
    nl += k;
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
      x.groups = A + s.c_groups;
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
      x.tune.stages = b->class_stages.empty() ? 0 : b->class_stages[c];
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
      // SMs no cluster fits on (not while timing candidates)
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
    HB_CK(launch_reduce_batch(sims, n, pre, b->totals, st));
    if (b->totals.red > 0) ++nl;
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
      // per class: the split-K depth (divisor 1, 2 or 4 of the chunk count)
      // and the cap on operand stages in shared memory (as many as fit, 5 or
      // 3: fewer leave more of the SM's memory to the L1 cache of the beam
      // gathers), each candidate's fused launch timed on this batch (the
      // second of two runs), the fastest kept
      b->class_stages.assign(b->classes.size(), 0);
      std::vector<int> best_div(b->classes.size(), 1), best_st(b->classes.size(), 0);
      std::vector<float> best_ms(b->classes.size(), 1e30f);
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        r = HV_ERR_CUDA;
        break;
      }
      for (int div : {1, 2, 4}) {
        b->class_nchunk_div.assign(b->classes.size(), div);
        layout(b);
        r = allocate(b);
        if (r == HV_OK) r = enqueue(b, st);  // preparation for this layout
        for (size_t c = 0; c < b->classes.size() && r == HV_OK; ++c) {
          for (int stages : {0, 5, 3}) {
            b->class_stages[c] = stages;
            float ms = 0.f;
            for (int rep = 0; rep < 2 && r == HV_OK; ++rep) {
              cudaEventRecord(e0, st);
              r = enqueue(b, st, (int)c);
              cudaEventRecord(e1, st);
              cudaEventSynchronize(e1);
              cudaEventElapsedTime(&ms, e0, e1);
            }
            // a candidate whose device-side waits gave up is never chosen,
            // and its flag does not carry over to the batch's own runs
            int flag = 0;
            if (r == HV_OK &&
                (cudaMemcpyAsync(&flag, b->d_err, sizeof(int), cudaMemcpyDeviceToHost, st) !=
                     cudaSuccess ||
                 cudaStreamSynchronize(st) != cudaSuccess))
              r = HV_ERR_CUDA;
            if (flag) {
              cudaMemsetAsync(b->d_err, 0, sizeof(int), st);
              ms = 1e30f;
            }
            if (r == HV_OK && ms < best_ms[c]) {
              best_ms[c] = ms;
              best_div[c] = div;
              best_st[c] = stages;
            }
          }
          b->class_stages[c] = 0;
        }
        if (r != HV_OK) break;
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      if (r != HV_OK) break;
      b->class_nchunk_div = best_div;
      b->class_stages = best_st;
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
    if (flag == 2 || flag == 3) return flag == 2 ? HV_ERR_ARG : HV_ERR_UNSUPPORTED;
    hv_context_set_error(b->ctx, "a device-side wait of the batch gave up; results of the "
                                 "last launch are invalid");
    return HV_ERR_TIMEOUT;
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
