// hv_tc.cu -- the fused tensor-core form of the hot path (sm_103a).
//
// One persistent kernel replaces the reference's per-chunk sequence
// SGEMM rotation -> SGEMM delay -> InterpolateBeam -> MeasEq -> CGEMM
// (hera_gpu/vis.py:224-250).  Phasors v[a, s] never leave the SM: they are
// generated straight into shared memory as split-BF16 operand tiles and
// contracted on the tensor cores (tcgen05.mma, FP32 accumulators in TMEM).
//
// Work decomposition
//   Antennas are cut into blocks of 128 (the MMA M).  The upper triangle of
//   block pairs (I <= J) is partitioned into groups of at most two pairs
//   that share their row block: (I, J) and (I, J + 1), and the pairs that
//   end a row on the last block, (I, nb - 1), taken transposed as
//   (nb - 1, I) below the diagonal so that they share the row block nb - 1
//   (their epilogue writes the conjugate back above it).  A group touches
//   at most three blocks ("slots") and runs as ONE MMA of N up to 256 per
//   K-step: the column blocks sit side by side in shared memory, so the row
//   block's operand is read once for both pairs.  Its accumulators -- Re V
//   in TMEM columns [0, 256), Im V in [256, 512) -- fill the 512 columns.
//   A work item is (time, frequency, source chunk, group); in cluster mode
//   (2-8 groups: 129-640 antennas) an item is (time, frequency, chunk) for a
//   thread-block cluster of one CTA per group, and each antenna block is
//   generated once per cluster, by the CTA that owns it, and pushed to the
//   peers that also use it.  A persistent grid of one CTA (or cluster) per
//   SM claims items at run time from a device counter.  Each item's partial
//   sum over its source chunk goes to HBM and a separate kernel reduces the
//   chunks in a fixed order (deterministic split-K over sources).
//
// Pipeline inside a CTA (split BF16: 12 + 3 warps; FP16 + FP8: 16 + 3)
//   generator warps  phasor generators, in teams that take stages in turn:
//                 for each (slot, antenna row, unit of 8 sources) the
//                 bilinear beam (4 coalesced gathers: lanes are antennas),
//                 the phase in cycles reduced exactly in FP32
//                 (phase_cycles32), sincos, v = A sqrt(I) e^{2 pi i phi},
//                 the split of v, stored to the canonical K-major
//                 128-byte-swizzled UMMA layout.  Every TC_FLUSH_SOURCES
//                 sources of an item, and after its last stage, they drain
//                 TMEM into the item's partial buffer (epilogue).
//   next warp     TMA producer: each stage's source records, one 2-D
//                 cp.async.bulk.tensor into shared memory.  Its first thread
//                 (in cluster mode, rank 0's) claims the items into a ring
//                 of item indices in shared memory that every role of every
//                 CTA of the cluster reads.
//   next warp     MMA issuer (one thread) and TMEM owner.
//   last warp     cluster mode: pushes this CTA's tiles to peer CTAs.
//
// Operand layout of one stage (16 sources): one tile per slot, the slots'
// tiles side by side (16 KB each: 128 rows x 128 bytes, K = 64 BF16 per
// antenna row), within a row the K chunks of 16 bytes
//   [Re hi s0-7, Re hi s8-15, Im hi s0-7, Im hi s8-15,
//    Re lo s0-7, Re lo s8-15, Im lo s0-7, Im lo s8-15]
//   so each MMA K-step (16 elements) holds the real or the imaginary parts
//   of the hi or the lo halves of the 16 sources, and per split product:
//     ReV += ReA ReB^T + ImA ImB^T,   ImV += ImA ReB^T - ReA ImB^T
//   (V[a,b] = sum_s v_a conj(v_b)); the minus sign is the instruction
//   descriptor's negate-A bit.  Split BF16 keeps hi*hi + hi*lo + lo*hi.
//
// Second form (kForm = 1, HV_METHOD_TC_FP16): FP16 hi parts and FP8 (E4M3)
// cross terms.  Per (time, frequency) slice the phasors are scaled by a power
// of two c so that |X| = |c v| <= 256 (c from a bound of the slice's largest
// |A| sqrt(I), tc_slice_bound_kernel), and split X = H + L with H the FP16
// rounding of X (11 significant bits) and L = X - H exact in FP32.  Then
//   X_a conj(X_b) ~ H_a conj(H_b) + e4m3(X_a) conj(e4m3(L_b))
//                                 + e4m3(L_a) conj(e4m3(X_b)),
// the first product on kind::f16, the two cross terms on kind::f8f6f4 (FP8
// runs at twice the FP16 rate), all into the same FP32 accumulators; the
// epilogue multiplies by 1/c^2 (exact).  A stage is 32 sources, with two
// tiles per slot (16 KB each, 128-byte rows):
//   FP16 tile  [Re H s0-31 | Im H s0-31]                  (64 B + 64 B)
//   FP8 tile   [Re X8 | Im X8 | Re L8 | Im L8], s0-31 each  (4 x 32 B)
// and 16 MMAs per group and stage (8 FP16 of K = 16, 8 FP8 of K = 32): the
// tensor-pipe time of 8 K = 16 BF16 MMAs per 16 sources, against 12 for
// split BF16.  Operand rounding costs about 1e-5 of relative error (3-bit
// mantissas on terms 2^-11 of the product).
//
// Every wait on an mbarrier is bounded in time; on expiry the kernel raises
// an error flag, lets in-flight copies and MMAs land (again bounded), frees
// TMEM and returns, so the host sees HV_ERR_TIMEOUT instead of a hung GPU.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "hv_internal.cuh"
#include "hv_kernels.h"

namespace hv {

constexpr int TC_ROWS = 128;          // antennas per block = MMA M
constexpr int TC_SLOT = 16384;        // one operand tile: 128 rows x 128 B
// Sources per stage: 16 for split BF16 (one tile per slot: hi and lo of 16
// sources), 32 for FP16 + FP8 (two tiles per slot, see above).
// Record stages: at least the operand stages (TC_MAX_STAGES), which makes
// every phase-parity wait on a record barrier exact (see the generators).
constexpr int TC_NREC_ALL = 8;
template <int kForm> struct TcForm;
template <> struct TcForm<0> {
  static constexpr int KS = 16, TILES = 1, NREC = TC_NREC_ALL;
};
template <> struct TcForm<1> {
  static constexpr int KS = 32, TILES = 2, NREC = TC_NREC_ALL;
};
constexpr int TC_KS_MAX = 32;
// Record stages: more than operand stages (they are small), so the TMA
// producer runs further ahead and a generator warp finds its next records
// loaded even while slower warps still hold earlier stages.

// Warp layout of each form.  The SM's four schedulers each hold a quarter
// of the block's warps, and a scheduler's 16K-register file is shared by
// its warps.
//  * Split BF16: 12 generator warps + 3 service warps (15; at most 4 a
//    scheduler), so a thread may hold 128 registers; teams of 4 warps, one
//    thread per antenna row generating all 16 sources of it per stage, three
//    teams taking the stages in turn.  Measured against 16 generator warps
//    at 96 registers (teams of 8): 7% faster at 350 antennas x 1M sources.
//  * FP16 + FP8: 16 generator warps + 3 service (19; 96 registers), one team
//    of 16 per 32-source stage (four thread groups along the stage, one
//    unit of 8 sources each).  Only three of its 64 KB stages fit beside the
//    records, so a stage must be generated by every generator at once: with
//    12 warps in three teams it ran 10% slower.
// One-slot launches of up to 64 (32) antennas use teams of half (a
// quarter) the full team, enough for their rows.
template <int kForm> struct TcLayout;
template <> struct TcLayout<0> {
  static constexpr int GEN_WARPS = 12, TEAM = 4, NSG = 1;
};
template <> struct TcLayout<1> {
  static constexpr int GEN_WARPS = 16, TEAM = 16, NSG = 4;
};
template <int kForm> constexpr int tc_threads() { return TcLayout<kForm>::GEN_WARPS * 32 + 96; }
static_assert(((tc_threads<0>() / 32 + 3) / 4) * 32 * 128 <= 16384,
              "split BF16: at most 4 warps a scheduler at 128 registers");
constexpr int TC_MAX_STAGES = 8;
// Sources accumulated in TMEM before the sum is added to the item's split-K
// partial in global memory (FP32, round to nearest) and the accumulator
// starts again.  The tensor core's accumulation into TMEM loses a fraction
// of an ulp of the accumulated value per addition, always toward zero, so
// its error grows with the number of additions into one value: measured
// against the FP64 oracle at 350 antennas x 1M sources, the relative error
// of an autocorrelation summed over 16384 sources is -1e-4, over 1024
// sources -1.3e-5.  TC_FLUSH_SOURCES (a multiple of every stage size) per
// flush bound it.
#ifndef TC_FLUSH_SOURCES
#define TC_FLUSH_SOURCES 2048
#endif
static_assert(TC_MAX_STAGES <= TC_NREC_ALL, "record stages >= operand stages");
static_assert(TC_FLUSH_SOURCES % TC_KS_MAX == 0, "flush interval: whole stages of every form");
constexpr int TC_TMEM_COLS = 512;
constexpr int TC_SMEM_LIMIT = 227 * 1024;
// default limit of one wait: 10 s, far above any wait of a working launch
// (an item lasts milliseconds), so that a disturbance of the timer the
// waits read cannot end a healthy wait
constexpr unsigned long long TC_WAIT_NS = 10000000000ull;

constexpr int kErrTimeout = 1;
constexpr int kErrRange = 2;    // |U| beyond the exact range of rint_magic
constexpr int kErrLayout = 3;   // dynamic shared memory not 1024-byte aligned

constexpr int TC_MAX_CLUSTER = 8;

struct TcGroup {
  int npairs, nslots;
  int slot_block[3];
  int slot_rows[3];  // valid antenna rows of each slot's block
  int sa;            // slot of the row block (A operand); the column blocks (B) are slots 0, 1
  int n_mma;         // MMA N: 128 + the columns of slot 1 for two pairs, else those of slot 0
  int pI[2], pJ[2];  // row and column block of each pair; pI > pJ: computed below the diagonal
  int pN[2];         // valid columns of block pJ, rounded up to 16
  // Cluster mode (one CTA per group, cluster rank = group index): every
  // block is generated by exactly one CTA of the cluster and written into
  // the shared memory of each CTA whose group uses it.
  int nown;                            // slots generated here
  int own_slot[3];                     // ... which ones
  int ndst[3];                         // per owned slot: other CTAs it goes to
  int dst_rank[3][TC_MAX_CLUSTER - 1];
  int dst_slot[3][TC_MAX_CLUSTER - 1];
  int recv_slots;                      // slots pushed here by peers per stage
  int empty_count;                     // arrivals per stage on this CTA's smem_empty
  int commit_mask;                     // CTAs this CTA's MMA completion is signalled to
  int write_mask;                      // CTAs this CTA's generators write to (bit = rank)
};

// One simulation of a launch.  A launch runs the items of every simulation
// in its table; all of them share the record tensor (rows from rec_row0).
struct TcSim {
  const int* counts;      // [nt] sources above the horizon per time
  const Ucoef32* U;       // [nt][nf][Np]
  const float* beamT;     // [nf][PP][Np]
  const float* umax;      // [nt * nf] bound of |U|_1 per slice
  const float* sbound;    // [nt * nf] bound of |A| sqrt(I) per slice (FP16 + FP8 form)
  float* partial;         // [nt * nf][nchunk][2][Np][Np]
  const TcGroup* groups;  // [ngroups]
  long long item0;        // first item of this simulation in the launch
  int rec_row0;           // first record row of time 0
  int rec_stride;         // records per time (a multiple of 32)
  int nt, nf, Np, PP, dx, dy;
  int nchunk, chunk, ngroups;
};

// A launch of one simulation carries its entry in the kernel parameters
// (kTable = false: the fields are constant-bank operands and hold no
// registers in the generator loop); a batched launch reads the table in
// global memory.
struct TcParams {
  const TcSim* sims;
  TcSim one;
  int nsims;
  long long total_items;
  int nstages, max_slots;
  int* err;
  unsigned long long wait_ns;  // limit of one wait
  int stall;                   // fault injection: the first record copy is never issued
  // Items are claimed at run time from *claim (zero before the launch):
  //  kClaimCount  one counter of the launch's own items (total_items);
  //  kClaimFront  shared launch of one simulation, its cluster kernel: whole
  //               cluster items from the front of the packed word (high 32
  //               bits: cluster items taken), while none of their group
  //               items has been taken from the back;
  //  kClaimBack   the one-CTA kernel of that shared launch, on the SMs no
  //               cluster fits on: group items (cluster item x ngroups +
  //               group) from the back (low 32 bits: group items taken),
  //               down to the front's last claim.
  // Every item is computed exactly once, whichever kernel starts first.
  unsigned long long* claim;
  int claim_mode;
  long long group_items;  // shared launch: cluster items x ngroups
  int team_warps;  // generator warps per stage without clusters (a full team, or 1/2 or 1/4)
};
constexpr int kClaimCount = 0, kClaimFront = 1, kClaimBack = 2;
// Items a CTA has claimed ahead of its slowest role (the ring of item
// indices in shared memory).
constexpr int TC_ITEM_RING = 4;

// Read-only load of a pointer-valued field.
template <typename T>
__device__ __forceinline__ T* ldg_ptr(T* const* p) {
  return reinterpret_cast<T*>(__ldg(reinterpret_cast<const unsigned long long*>(p)));
}

// ------------------------------------------------------------ PTX helpers --
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
// try_wait with a suspend-time hint: a waiting thread sleeps in hardware
// until the phase completes or the hint (ns) elapses, instead of polling
// the barrier through the shared-memory pipe.
constexpr uint32_t kSuspendHintNs = 20000;
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity), "r"(kSuspendHintNs)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_try_cluster(uint32_t bar, uint32_t parity);

// Single-thread bounded wait (kCl: acquire at cluster scope, for barriers
// that threads of other CTAs arrive on).
template <bool kCl = false>
__device__ __forceinline__ bool wait1(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                      int* gerr, unsigned long long limit_ns) {
  const unsigned long long t0 = global_ns();
  for (uint32_t i = 0;; ++i) {
    if (kCl ? mbar_try_cluster(bar, parity) : mbar_try(bar, parity)) return true;
    if ((i & 63) == 63) {
      if (*abort_flag) return false;
      if (global_ns() - t0 > limit_ns) {
        *abort_flag = 1;
        atomicExch(gerr, kErrTimeout);
        return false;
      }
    }
  }
}

// Whole-warp bounded wait; the outcome is uniform across the warp.
template <bool kCl = false>
__device__ __forceinline__ bool wait_warp(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                          int* gerr, unsigned long long limit_ns) {
  const unsigned long long t0 = global_ns();
  for (uint32_t i = 0;; ++i) {
    const bool done = kCl ? mbar_try_cluster(bar, parity) : mbar_try(bar, parity);
    if (__all_sync(0xffffffffu, done)) return true;
    if (i >= 2) __nanosleep(64);  // leave issue slots to the MMA warp
    if ((i & 63) == 63) {
      int give_up = 0;
      if ((threadIdx.x & 31) == 0) {
        if (*abort_flag) {
          give_up = 1;
        } else if (global_ns() - t0 > limit_ns) {
          *abort_flag = 1;
          atomicExch(gerr, kErrTimeout);
          give_up = 1;
        }
      }
      if (__shfl_sync(0xffffffffu, give_up, 0)) return false;
    }
  }
}

// Bounded wait used while shutting down: ignores the abort flag so that
// copies and MMAs already in flight still land before TMEM is released.
__device__ __forceinline__ void wait_drain(uint32_t bar, uint32_t parity, int* gerr,
                                           unsigned long long limit_ns) {
  const unsigned long long t0 = global_ns();
  for (uint32_t i = 0;; ++i) {
    if (mbar_try(bar, parity)) return;
    if ((i & 63) == 63 && global_ns() - t0 > limit_ns) {
      atomicExch(gerr, kErrTimeout);
      return;
    }
  }
}

// cluster-scope variants (distributed shared memory)
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t map_to_rank(uint32_t saddr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
  return r;
}
__device__ __forceinline__ void sts128_cluster(uint32_t addr, uint4 v) {
  asm volatile("st.shared::cluster.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(v.x),
               "r"(v.y), "r"(v.z), "r"(v.w)
               : "memory");
}
__device__ __forceinline__ void st_cluster_b64(uint32_t addr, long long v) {
  asm volatile("st.shared::cluster.b64 [%0], %1;" ::"r"(addr), "l"(v) : "memory");
}
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t remote_bar) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(remote_bar)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_cluster(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2, %3;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity), "r"(kSuspendHintNs)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void fence_async_smem_cluster() {
  asm volatile("fence.proxy.async.shared::cluster;" ::: "memory");
}
__device__ __forceinline__ void mma_commit_multicast(uint32_t bar, uint16_t mask) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64"
      " [%0], %1;" ::"r"(bar), "h"(mask)
      : "memory");
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::
                   : "memory");
}

// Copy engine push of `bytes` from this CTA's shared memory to a peer's
// (dst and its barrier given as cluster addresses); completion is signalled
// on the peer's barrier as transaction bytes.
__device__ __forceinline__ void bulk_push(uint32_t dst_cluster, uint32_t src_cta, uint32_t bytes,
                                          uint32_t bar_cluster) {
  asm volatile(
      "cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(dst_cluster), "r"(src_cta), "r"(bytes), "r"(bar_cluster)
      : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, uint32_t bar,
                                            int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4}], [%2];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(x), "r"(y)
      : "memory");
}

// Shared-memory matrix descriptor, K-major with the 128-byte swizzle: 8-row
// atoms of 1024 bytes (stride byte offset), descriptor version 1 (sm_100
// family).  The high word is the same for every operand; the low word holds
// the start address (>> 4) and the leading byte offset (unused for this
// layout).  Advancing along K by 32 bytes adds 2 to the low word.
constexpr uint32_t kDescHi = (1024u >> 4) | (1u << 14) | (2u << 29);
__device__ __forceinline__ uint32_t desc_lo(uint32_t saddr) {
  return ((saddr & 0x3FFFFu) >> 4) | (1u << 16);
}

// Instruction descriptor: D F32, A and B K-major, M = 128, N = n; the A/B
// type code is 1 for BF16 (kind::f16) and 0 for FP16 (kind::f16) or E4M3
// (kind::f8f6f4).
__device__ __forceinline__ uint32_t idesc_mma(int n, bool negate_a, uint32_t ab_type) {
  uint32_t d = (1u << 4) | (ab_type << 7) | (ab_type << 10);
  d |= (uint32_t)(n >> 3) << 17;
  d |= (uint32_t)(TC_ROWS >> 4) << 24;
  if (negate_a) d |= 1u << 13;
  return d;
}
__device__ __forceinline__ uint32_t idesc_bf16(int n, bool negate_a) {
  return idesc_mma(n, negate_a, 1u);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint32_t a_lo, uint32_t b_lo,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n .reg .b64 da, db;\n setp.ne.b32 p, %5, 0;\n"
      " mov.b64 da, {%1, %3};\n mov.b64 db, {%2, %3};\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], da, db, %4, p;\n}\n" ::"r"(d_tmem),
      "r"(a_lo), "r"(b_lo), "r"(kDescHi), "r"(idesc), "r"(accumulate)
      : "memory");
}

// The 12 MMAs of one group and one stage (16 sources): for each split
// product (hi hi, hi lo, lo hi),
//   ReV += ReA ReB + ImA ImB,   ImV += ImA ReB - ReA ImB,
// with B the group's column blocks side by side (N up to 256).  a, b:
// descriptor low words of the row block's tile and of the first column
// block's tile; along K, Re hi, Im hi, Re lo, Im lo are 32 bytes (2
// descriptor units) apart.  first: the stage opens the item.
__device__ __forceinline__ void issue_group(uint32_t d_re, uint32_t a, uint32_t b, uint32_t idp,
                                            uint32_t idn, bool first) {
  const uint32_t d_im = d_re + 256;
#pragma unroll
  for (int pr = 0; pr < 3; ++pr) {
    const uint32_t aa = a + (pr == 2 ? 4u : 0u), bb = b + (pr == 1 ? 4u : 0u);  // lo: 64 B on
    const uint32_t acc = (first && pr == 0) ? 0u : 1u;
    mma_bf16(d_re, aa, bb, idp, acc);            // Re Re
    mma_bf16(d_re, aa + 2u, bb + 2u, idp, 1u);   // Im Im
    mma_bf16(d_im, aa + 2u, bb, idp, acc);       // Im Re
    mma_bf16(d_im, aa, bb + 2u, idn, 1u);        // -Re Im
  }
}

// kind::f8f6f4 with E4M3 operands (K = 32 per instruction).
__device__ __forceinline__ void mma_e4m3(uint32_t d_tmem, uint32_t a_lo, uint32_t b_lo,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n .reg .b64 da, db;\n setp.ne.b32 p, %5, 0;\n"
      " mov.b64 da, {%1, %3};\n mov.b64 db, {%2, %3};\n"
      " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], da, db, %4, p;\n}\n" ::"r"(d_tmem),
      "r"(a_lo), "r"(b_lo), "r"(kDescHi), "r"(idesc), "r"(accumulate)
      : "memory");
}

// The 16 MMAs of one group and one 32-source stage of the FP16 + FP8 form.
// a16/b16: descriptor low words of the row block's and the column blocks'
// FP16 tiles (K chunks of 32 bytes: Re s0-15, Re s16-31, Im s0-15, Im s16-31
// at +0, +2, +4, +6); a8/b8: the FP8 tiles (Re X8, Im X8, Re L8, Im L8 at
// +0, +2, +4, +6).  The FP16 and E4M3 instruction descriptors coincide.
__device__ __forceinline__ void issue_group_f16f8(uint32_t d_re, uint32_t a16, uint32_t b16,
                                                  uint32_t a8, uint32_t b8, uint32_t idp,
                                                  uint32_t idn, bool first) {
  const uint32_t d_im = d_re + 256;
#pragma unroll
  for (uint32_t h = 0; h < 4; h += 2) {  // source halves s0-15, s16-31
    const uint32_t acc = (first && h == 0) ? 0u : 1u;
    mma_bf16(d_re, a16 + h, b16 + h, idp, acc);              // Re Re
    mma_bf16(d_re, a16 + 4u + h, b16 + 4u + h, idp, 1u);     // Im Im
    mma_bf16(d_im, a16 + 4u + h, b16 + h, idp, acc);         // Im Re
    mma_bf16(d_im, a16 + h, b16 + 4u + h, idn, 1u);          // -Re Im
  }
#pragma unroll
  for (int pr = 0; pr < 2; ++pr) {  // X8 (a) x L8 (b), then L8 (a) x X8 (b)
    const uint32_t xa = pr == 0 ? 0u : 4u, yb = pr == 0 ? 4u : 0u;
    mma_e4m3(d_re, a8 + xa, b8 + yb, idp, 1u);               // Re Re
    mma_e4m3(d_re, a8 + xa + 2u, b8 + yb + 2u, idp, 1u);     // Im Im
    mma_e4m3(d_im, a8 + xa + 2u, b8 + yb, idp, 1u);          // Im Re
    mma_e4m3(d_im, a8 + xa, b8 + yb + 2u, idn, 1u);          // -Re Im
  }
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Adds to global memory without returning the old value (the addition is
// done at L2, rounded to nearest); one thread's additions and stores to an
// address take effect in program order.
__device__ __forceinline__ void red_add(float* p, float v) {
  asm volatile("red.global.add.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}
__device__ __forceinline__ void red_add4(float4* p, float4 v) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(v.x), "f"(v.y),
               "f"(v.z), "f"(v.w)
               : "memory");
}

__device__ __forceinline__ void sts64(uint32_t addr, uint2 v) {
  asm volatile("st.shared.v2.b32 [%0], {%1, %2};" ::"r"(addr), "r"(v.x), "r"(v.y) : "memory");
}

__device__ __forceinline__ void sts128(uint32_t addr, uint4 v) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(v.x), "r"(v.y),
               "r"(v.z), "r"(v.w)
               : "memory");
}

// rint for |x| < 2^22 with two FP32 adds (FMA pipe) instead of FRND.
__device__ __forceinline__ float rint_magic(float x) {
  return __fsub_rn(__fadd_rn(x, 12582912.0f), 12582912.0f);
}

// phase_cycles32 (hv_internal.cuh) with rint_magic: |U . s| < 2^21 cycles
// is checked on the host before launch.
__device__ __forceinline__ float phase_exact(const Ucoef32& u, float sx, float sy, float sz) {
  const float p0 = __fmul_rn(u.hx, sx);
  const float p1 = __fmul_rn(u.hy, sy);
  const float p2 = __fmul_rn(u.hz, sz);
  const float e0 = fmaf(u.hx, sx, -p0);
  const float e1 = fmaf(u.hy, sy, -p1);
  const float e2 = fmaf(u.hz, sz, -p2);
  const float r0 = __fsub_rn(p0, rint_magic(p0));
  const float r1 = __fsub_rn(p1, rint_magic(p1));
  const float r2 = __fsub_rn(p2, rint_magic(p2));
  const float lo = fmaf(u.lx, sx, fmaf(u.ly, sy, fmaf(u.lz, sz, __fadd_rn(__fadd_rn(e0, e1), e2))));
  const float ph = __fadd_rn(__fadd_rn(r0, r1), __fadd_rn(r2, lo));
  return __fsub_rn(ph, rint_magic(ph));
}

// Eight floats -> BF16 hi parts and BF16 residuals (v - hi), packed in
// pairs (lower K index in the low half-word).
__device__ __forceinline__ uint32_t bf16x2_bits(float lo, float hi) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&h);
}
__device__ __forceinline__ void split_pack(const float* v, uint4& hi, uint4& lo) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    h[i] = bf16x2_bits(v[2 * i], v[2 * i + 1]);
    const float r0 = v[2 * i] - __uint_as_float(h[i] << 16);
    const float r1 = v[2 * i + 1] - __uint_as_float(h[i] & 0xffff0000u);
    l[i] = bf16x2_bits(r0, r1);
  }
  hi = make_uint4(h[0], h[1], h[2], h[3]);
  lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// Eight scaled phasor parts X -> their FP16 roundings H (packed in pairs,
// lower K index in the low half-word), and the E4M3 roundings (saturating)
// of X and of L = X - H (exact in FP32), packed four to a word.
__device__ __forceinline__ void split_f16_e4m3(const float* x, uint4& h16, uint2& x8,
                                               uint2& l8) {
  uint32_t h[4];
  uint32_t px[4], pl[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const __half2 hh = __floats2half2_rn(x[2 * i], x[2 * i + 1]);
    h[i] = *reinterpret_cast<const uint32_t*>(&hh);
    const float2 hf = __half22float2(hh);
    px[i] = __nv_cvt_float2_to_fp8x2(make_float2(x[2 * i], x[2 * i + 1]), __NV_SATFINITE,
                                     __NV_E4M3);
    pl[i] = __nv_cvt_float2_to_fp8x2(make_float2(x[2 * i] - hf.x, x[2 * i + 1] - hf.y),
                                     __NV_SATFINITE, __NV_E4M3);
  }
  h16 = make_uint4(h[0], h[1], h[2], h[3]);
  x8 = make_uint2(__byte_perm(px[0], px[1], 0x5410), __byte_perm(px[2], px[3], 0x5410));
  l8 = make_uint2(__byte_perm(pl[0], pl[1], 0x5410), __byte_perm(pl[2], pl[3], 0x5410));
}

// Scale of a slice of the FP16 + FP8 form: c = 2^k with c * bound <= 256
// (bound: the slice's largest |A| sqrt(I), or a bound of it), and 1 / c^2.
__device__ __forceinline__ void slice_scale(float bound, float& c, float& inv_c2) {
  int e = 0;  // bound <= 2^e
  const uint32_t b = __float_as_uint(bound);
  const int ex = (int)((b >> 23) & 0xffu);
  if (bound > 0.f && ex < 255) {
    e = ex == 0 ? -126 : ex - 127 + ((b & 0x7fffffu) ? 1 : 0);
  }
  const int k = max(-60, min(60, 8 - e));
  c = __uint_as_float((uint32_t)(127 + k) << 23);
  inv_c2 = __uint_as_float((uint32_t)(127 - 2 * k) << 23);
}

// Phasors of 8 consecutive records (one unit) for one antenna: v = A sqrt(I)
// e^{2 pi i phi}.  Record 0's direction is the unit's reference; its pad word
// holds the largest |s - s_ref|_1 of the unit (tc_relative_kernel), its sign
// bit set when all eight sources share a beam pixel (then the four corners
// are loaded once for the unit).  When
// that is below dlim = 32 / max_a |U_a|_1 for this slice, the phases are
// U . s_ref (exact) + U . (s - s_ref), the second term below 32 cycles and
// so rounded to a few 1e-6 cycles in FP32 (worst case ~8e-6 cycles, 5e-5
// rad; the BF16 hi/lo operands carry 16 significant bits, 1.5e-5);
// otherwise every phase is computed exactly.
// All lanes read the same records, so the branch does not diverge.  Padding
// records have zero amplitude.  beam_a: the antenna's column of the
// transposed beam.
template <bool kNear, bool kOnePixel>
__device__ __forceinline__ void gen_unit_path(const SrcRec32* rec, const Ucoef32& uc,
                                              const float* beam_a, int Np, int dx, int dy,
                                              float4 ref, float ph_ref, float csc, float* rv,
                                              float* iv) {
  // one pixel for the unit: its corners as c00 + fx d1 + fy (d2 + fx d3),
  // the bilinear interpolant with the differences formed once per unit
  float c00 = 0.f, d1 = 0.f, d2 = 0.f, d3 = 0.f;
  if (kOnePixel) {
    const float* bp = beam_a + (size_t)__float_as_int(reinterpret_cast<const float4*>(rec)[1].x) * Np;
    c00 = __ldg(bp);
    const float c01 = __ldg(bp + (size_t)dx * Np);
    const float c10 = __ldg(bp + (size_t)dy * Np);
    const float c11 = __ldg(bp + (size_t)(dx + dy) * Np);
    d1 = c01 - c00;
    d2 = c10 - c00;
    d3 = (c11 - c10) - d1;
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const float4* rp = reinterpret_cast<const float4*>(rec + q);
    const float4 ra = rp[0], rb = rp[1];  // sx sy sz amp | pix fx fy -
    float A;
    if (kOnePixel) {
      A = fmaf(rb.z, fmaf(rb.y, d3, d2), fmaf(rb.y, d1, c00));
    } else {
      const float* bp = beam_a + (size_t)__float_as_int(rb.x) * Np;
      const float b00 = __ldg(bp);
      const float b01 = __ldg(bp + (size_t)dx * Np);
      const float b10 = __ldg(bp + (size_t)dy * Np);
      const float b11 = __ldg(bp + (size_t)(dx + dy) * Np);
      A = lerp(lerp(b00, b01, rb.y), lerp(b10, b11, rb.y), rb.z);
    }
    float ph;
    if (!kNear) {
      ph = phase_exact(uc, ra.x, ra.y, ra.z);
    } else if (q == 0) {
      ph = ph_ref;
    } else {
      const float ex = __fsub_rn(ra.x, ref.x), ey = __fsub_rn(ra.y, ref.y),
                  ez = __fsub_rn(ra.z, ref.z);
      ph = fmaf(uc.hx, ex, fmaf(uc.hy, ey, fmaf(uc.hz, ez, ph_ref)));
      ph = __fsub_rn(ph, rint_magic(ph));
    }
    // the hardware sin/cos on [-pi, pi] (absolute error ~4e-7) is ample for
    // BF16 operands
    float sn, cs;
    __sincosf(6.28318530717958648f * ph, &sn, &cs);
    const float amp = A * (ra.w * csc);
    rv[q] = amp * cs;
    iv[q] = amp * sn;
  }
}

// csc: the slice's scale (1 for split BF16; a power of two, so exact).
__device__ __forceinline__ void gen_unit(const SrcRec32* rec, const Ucoef32& uc,
                                         const float* beam_a, int Np, int dx, int dy, float dlim,
                                         float csc, float* rv, float* iv) {
  const float4* rp0 = reinterpret_cast<const float4*>(rec);
  const float4 q0a = rp0[0], q0b = rp0[1];
  const int flags = __float_as_int(q0b.w);
  const bool one_pixel = flags < 0;
  const bool near = __int_as_float(flags & 0x7fffffff) <= dlim;
  if (near) {
    const float ph_ref = phase_exact(uc, q0a.x, q0a.y, q0a.z);
    if (one_pixel) gen_unit_path<true, true>(rec, uc, beam_a, Np, dx, dy, q0a, ph_ref, csc, rv, iv);
    else gen_unit_path<true, false>(rec, uc, beam_a, Np, dx, dy, q0a, ph_ref, csc, rv, iv);
  } else {
    gen_unit_path<false, false>(rec, uc, beam_a, Np, dx, dy, q0a, 0.f, csc, rv, iv);
  }
}

// ------------------------------------------------------------- the kernel --
// Position of a global stage counter in the ring of NS operand stages (slot
// and phase parity), moved forward without dividing by the runtime NS.
struct StageRing {
  uint32_t s = 0, ph = 0;
  __device__ __forceinline__ void advance(uint32_t by, uint32_t ns) {  // by <= ns
    s += by;
    if (s >= ns) {
      s -= ns;
      ph ^= 1u;
    }
  }
};
static_assert((TcForm<0>::NREC & (TcForm<0>::NREC - 1)) == 0 &&
                  (TcForm<1>::NREC & (TcForm<1>::NREC - 1)) == 0,
              "the record ring is indexed by masks");

// The next item of this CTA (or cluster), or -1 when the launch's items are
// all taken (see TcParams::claim).
__device__ __forceinline__ long long claim_item(const TcParams& p) {
  if (p.claim_mode == kClaimCount) {
    const unsigned long long x = atomicAdd(p.claim, 1ull);
    return x < (unsigned long long)p.total_items ? (long long)x : -1;
  }
  const unsigned long long C = (unsigned long long)p.one.ngroups;
  const unsigned long long G = (unsigned long long)p.group_items;
  volatile unsigned long long* w = p.claim;
  for (;;) {
    const unsigned long long old = *w;
    const unsigned long long f = old >> 32, b = old & 0xffffffffull;
    if (p.claim_mode == kClaimFront) {
      if ((f + 1) * C + b > G) return -1;  // its groups reach the back's claims
      if (atomicCAS(p.claim, old, old + (1ull << 32)) == old) return (long long)f;
    } else {
      if (f * C + b >= G) return -1;       // the front took the rest
      if (atomicCAS(p.claim, old, old + 1ull) == old) return (long long)(G - 1 - b);
    }
  }
}

struct ItemInfo {
  const TcSim* sim;
  int g, k, tl, f, sl;
  int s0, s1, nst;
};

// Item it -> (simulation, group, chunk, slice).  Without clusters an item is
// one group of one (slice, chunk); in cluster mode an item is a (slice,
// chunk) and every CTA of the cluster takes its own group (its rank).
// Field f of the item's simulation (d: its ItemInfo).
#define SIM_I(d, f) (kTable ? __ldg(&(d).sim->f) : p.one.f)
#define SIM_P(d, f) (kTable ? ldg_ptr(&(d).sim->f) : p.one.f)

template <bool kCluster, bool kTable, int kKS>
__device__ __forceinline__ bool decode_item(const TcParams& p, long long it, int rank,
                                            ItemInfo& d) {
  long long rest = it;
  if (kTable) {
    int lo = 0, hi = p.nsims - 1;  // last simulation with item0 <= it
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(&p.sims[mid].item0) <= it) lo = mid;
      else hi = mid - 1;
    }
    d.sim = p.sims + lo;
    rest -= __ldg(&d.sim->item0);
  }
  // A simulation's items enumerate only the source chunks that hold sources
  // above the horizon: per time t, chunks k < ceil(count_t / chunk), each for
  // every frequency (and, without clusters, every group), chunk-major so
  // that the short last chunk of a time comes last.  Item indices past the
  // last such chunk (the host counts every chunk) decode to nothing.
  const int ngroups = SIM_I(d, ngroups), nf = SIM_I(d, nf), nt = SIM_I(d, nt);
  const int chunk = SIM_I(d, chunk);
  const int* counts = SIM_P(d, counts);
  if (kCluster) {
    d.g = rank;
  } else {
    d.g = (int)(rest % ngroups);
    rest = rest / ngroups;
  }
  int t = 0, cnt = 0;
  for (; t < nt; ++t) {
    cnt = __ldg(counts + t);
    const long long n_t = (long long)((cnt + chunk - 1) / chunk) * nf;
    if (rest < n_t) break;
    rest -= n_t;
  }
  if (t >= nt) return false;
  d.k = (int)(rest / nf);
  d.f = (int)(rest % nf);
  d.tl = t;
  d.sl = t * nf + d.f;
  d.s0 = d.k * chunk;
  d.s1 = min(d.s0 + chunk, cnt);
  d.nst = (d.s1 - d.s0 + kKS - 1) / kKS;
  return true;
}

// One CTA per SM; the launch bounds give each form's register budget (split
// BF16: 15 warps, 128 registers a thread; FP16 + FP8: 19 warps, 96).
template <bool kCluster, bool kTable, int kForm>
__global__ void __launch_bounds__(tc_threads<kForm>(), 1)
tc_vis_kernel(const __grid_constant__ CUtensorMap rec_map, const __grid_constant__ TcParams p) {
  // warp roles: generators, then the TMA producer, the MMA issuer and the
  // cluster-mode pusher of tiles to peer CTAs
  constexpr int TC_GEN_WARPS = TcLayout<kForm>::GEN_WARPS;
  constexpr int TC_GEN_THREADS = TC_GEN_WARPS * 32;
  constexpr int TC_PRODUCER_WARP = TC_GEN_WARPS;
  constexpr int TC_MMA_WARP = TC_GEN_WARPS + 1;
  constexpr int TC_PUSH_WARP = TC_GEN_WARPS + 2;
  constexpr int KS = TcForm<kForm>::KS;         // sources per stage
  constexpr int TILES = TcForm<kForm>::TILES;   // tiles per slot per stage
  constexpr int REC = KS * 32;                  // record bytes per stage
  constexpr int FLUSH = TC_FLUSH_SOURCES / KS;  // stages per accumulator flush
  constexpr int TC_NREC = TcForm<kForm>::NREC;  // record stages
  // generator warps per stage in cluster mode (compile-time there; launches
  // without clusters take theirs from the parameters)
  constexpr int CL_TEAM = TcLayout<kForm>::TEAM;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // The operand tiles need a 1024-byte aligned base (the 128-byte swizzle
  // atoms); the launch reserves no slack for aligning it, which keeps the
  // request within a smaller shared-memory carve-out.  A base that is not
  // aligned is reported (HV_ERR_UNSUPPORTED on the host) before any shared
  // memory is touched -- every CTA sees the same offset and returns.
  if ((smem_u32(smem_raw) & 1023u) != 0u) {
    if (threadIdx.x == 0) atomicExch(p.err, kErrLayout);
    return;
  }
  uint8_t* smem = smem_raw;
  const int NS = p.nstages;
  const uint32_t op_base = smem_u32(smem);
  // a stage: the FP16 / split-BF16 tiles of every slot side by side, then
  // (FP16 + FP8 form) the FP8 tiles of every slot side by side
  const uint32_t tile8_off = (uint32_t)p.max_slots * TC_SLOT;
  const uint32_t stage_bytes = (uint32_t)TILES * tile8_off;
  uint8_t* rec_smem = smem + (size_t)NS * stage_bytes;
  const uint32_t rec_base = smem_u32(rec_smem);
  uint64_t* bars = reinterpret_cast<uint64_t*>(rec_smem + (size_t)TC_NREC * REC);
  const uint32_t bar0 = smem_u32(bars);
  // barrier addresses
  // record stages r < TC_NREC, operand stages s < NS
  auto rec_full = [&](int r) { return bar0 + 8u * r; };
  auto rec_empty = [&](int r) { return bar0 + 8u * (TC_NREC + r); };
  const uint32_t sbar0 = bar0 + 8u * (2 * TC_NREC);
  auto smem_full = [&](int s) { return sbar0 + 8u * s; };
  auto smem_empty = [&](int s) { return sbar0 + 8u * (NS + s); };
  auto gen_done = [&](int s) { return sbar0 + 8u * (2 * NS + s); };
  const uint32_t acc_full = sbar0 + 8u * (3 * NS);
  const uint32_t acc_empty = acc_full + 8;
  const uint32_t drain = acc_full + 16;
  // ring of claimed item indices: written by the claiming thread (in
  // cluster mode rank 0's, into every CTA of the cluster), read by every
  // role; item_empty of the claiming CTA counts the reads of all CTAs
  const uint32_t ibar0 = acc_full + 24;
  auto item_full = [&](int k) { return ibar0 + 8u * k; };
  auto item_empty = [&](int k) { return ibar0 + 8u * (TC_ITEM_RING + k); };
  long long* item_ring = reinterpret_cast<long long*>(bars + 2 * TC_NREC + 3 * NS + 3 +
                                                      2 * TC_ITEM_RING);
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(item_ring + TC_ITEM_RING);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_holder + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rank = kCluster ? (int)cluster_rank() : 0;
  // cluster mode: every simulation of the launch has the same group layout
  // (one group per CTA of the cluster), so its barrier counts are common
  const int csize = kCluster ? (kTable ? (int)__ldg(&p.sims[0].ngroups) : p.one.ngroups) : 1;
  const TcGroup* groups0 = kTable ? ldg_ptr(&p.sims[0].groups) : p.one.groups;
  const TcGroup* mine = groups0 + rank;
  // cluster mode: operand bytes this CTA receives from peers per stage
  const uint32_t recv_bytes =
      kCluster ? (uint32_t)__ldg(&mine->recv_slots) * (uint32_t)(TILES * TC_SLOT) : 0u;
  // cluster mode: does this CTA generate any block?
  const int nown = kCluster ? __ldg(&mine->nown) : 0;
  const bool generates = !kCluster || nown > 0;
  if (threadIdx.x == 0) {
    // arrivals per stage on smem_full: one per generator warp of the team
    // (if this CTA generates) and, in cluster mode, the MMA thread's arming
    // of the bytes its peers push
    const int team_warps = kCluster ? CL_TEAM : p.team_warps;
    const int full_count = (generates ? team_warps : 0) + (recv_bytes ? 1 : 0);
    const int empty_count = kCluster ? mine->empty_count : 1;
    for (int r = 0; r < TC_NREC; ++r) {
      mbar_init(rec_full(r), 1);
      mbar_init(rec_empty(r), team_warps);
    }
    for (int s = 0; s < NS; ++s) {
      mbar_init(smem_full(s), full_count);
      mbar_init(smem_empty(s), empty_count);
      mbar_init(gen_done(s), team_warps);
    }
    mbar_init(acc_full, 1);
    mbar_init(acc_empty, TC_GEN_THREADS);
    mbar_init(drain, 1);
    // readers of each claimed item: every generator warp and the MMA thread
    // of every CTA, the pusher and (but for the claimer's own) the producer
    // of every generating CTA
    int readers = TC_GEN_WARPS + 1;
    if (kCluster && rank == 0) {
      readers = 0;
      for (int r = 0; r < csize; ++r) {
        const int gen_r = __ldg(&groups0[r].nown) > 0;
        readers += TC_GEN_WARPS + 1 + gen_r + (r != 0 && gen_r);
      }
    }
    for (int k = 0; k < TC_ITEM_RING; ++k) {
      mbar_init(item_full(k), 1);
      mbar_init(item_empty(k), readers);
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    // the first round of every stage expects the peers' pushed tiles
    if (recv_bytes)
      for (int s = 0; s < NS; ++s) mbar_expect_tx(smem_full(s), recv_bytes);
  }
  if (warp == TC_MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_holder)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  // peers may arrive on our barriers only once every CTA has initialised them
  if (kCluster) cluster_sync_all();
  tc_fence_after();
  const uint32_t tmem = *tmem_holder;

  // The k-th item of this CTA, read from the ring by one thread (or a whole
  // warp, kWarp: every lane reads it), its slot then released to the
  // claiming CTA; false if a wait gave up.
  auto read_item = [&](uint32_t k, long long& it, auto warp_tag) -> bool {
    constexpr bool kWarp = decltype(warp_tag)::value;
    const int slot = (int)(k % TC_ITEM_RING);
    const uint32_t par = (k / TC_ITEM_RING) & 1;
    const bool got = kWarp ? wait_warp<kCluster>(item_full(slot), par, abort_flag, p.err, p.wait_ns)
                           : wait1<kCluster>(item_full(slot), par, abort_flag, p.err, p.wait_ns);
    if (!got) return false;
    it = *reinterpret_cast<volatile long long*>(item_ring + slot);
    if (!kWarp || lane == 0) {
      if (kCluster) mbar_arrive_cluster(map_to_rank(item_empty(slot), 0));
      else mbar_arrive(item_empty(slot));
    }
    return true;
  };
  using one_thread = std::integral_constant<bool, false>;
  using whole_warp = std::integral_constant<bool, true>;

  if (warp < TC_GEN_WARPS) {
    // ------------------------------------------------ phasor generators --
    const int tid = threadIdx.x;
    const int team_warps = kCluster ? CL_TEAM : p.team_warps;
    const int nteams = TC_GEN_WARPS / team_warps;
    const int team = warp / team_warps;  // takes the stages with gs % nteams == team
    uint32_t gs = 0, ic = 0;
    // this team's next stage (global counter) and its operand-ring position
    uint32_t my_gs = (uint32_t)team;
    StageRing ring;
    ring.advance((uint32_t)team, (uint32_t)NS);
    ItemInfo d;
    for (uint32_t k = 0;; ++k) {
      long long it;
      if (!read_item(k, it, whole_warp{}) || it < 0) break;
      if (!decode_item<kCluster, kTable, KS>(p, it, rank, d)) continue;
      const TcGroup* gp = SIM_P(d, groups) + d.g;
      const int Np = SIM_I(d, Np), dx = SIM_I(d, dx), dy = SIM_I(d, dy);
      const int g_nslots = __ldg(&gp->nslots), g_npairs = __ldg(&gp->npairs);
      const int g_rows0 = __ldg(&gp->slot_rows[0]), g_rows1 = __ldg(&gp->slot_rows[1]),
                g_rows2 = __ldg(&gp->slot_rows[2]);
      const int g_blk0 = __ldg(&gp->slot_block[0]), g_blk1 = __ldg(&gp->slot_block[1]),
                g_blk2 = __ldg(&gp->slot_block[2]);
      const Ucoef32* Us = SIM_P(d, U) + (size_t)d.sl * Np;
      const float umax_sl = __ldg(SIM_P(d, umax) + d.sl);
      if (umax_sl >= 4.0e6f && tid == 0) atomicExch(p.err, kErrRange);
      const float dlim = 32.0f / fmaxf(umax_sl, 1e-30f);
      const float* beam = SIM_P(d, beamT) + (size_t)d.f * SIM_I(d, PP) * Np;
      // the slice's scale (FP16 + FP8 form)
      float csc = 1.f, inv_c2 = 1.f;
      if (kForm == 1) slice_scale(__ldg(SIM_P(d, sbound) + d.sl), csc, inv_c2);
      // the slots this CTA fills: all of its group's (no clusters) or the
      // ones it owns (cluster mode)
      const int nfill = kCluster ? nown : g_nslots;
      // this thread's units (fixed for the item): antenna row `row` and the
      // units of 8 sources [sg * upt, sg * upt + upt) of its team's stages,
      // in each slot it fills
      // a team covers its rows (128, or fewer for the small teams of
      // one-slot launches) with NSG thread groups along the stage
      constexpr int NSG = TcLayout<kForm>::NSG;
      constexpr int UPT = (KS / 8) / NSG;  // units per thread per stage
      static_assert(UPT >= 1 && UPT * NSG * 8 == KS, "a stage's units split evenly");
      const int tt = tid % (team_warps * 32);
      const int nrows = kCluster ? TC_ROWS : team_warps * 32 / NSG;
      const int row = tt % nrows, sg = tt / nrows;
      int u_slot[3], u_a[3];
      bool u_ok[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const int slot = kCluster ? __ldg(&gp->own_slot[i]) : i;
        u_slot[i] = slot;
        const int srows = slot == 0 ? g_rows0 : (slot == 1 ? g_rows1 : g_rows2);
        const int sblk = slot == 0 ? g_blk0 : (slot == 1 ? g_blk1 : g_blk2);
        u_ok[i] = i < nfill && row < srows;
        u_a[i] = sblk * TC_ROWS + row;
      }
      // the phase coefficients of the first unit's antenna, fixed for the item
      Ucoef32 uc0 = {};
      if (u_ok[0]) uc0 = Us[u_a[0]];
      const int r8 = row & 7;
      const uint32_t rowoff = (uint32_t)(row >> 3) * 1024u + (uint32_t)r8 * 128u;
      bool ok = true;
      // before reading the accumulator of a flush, generate the first
      // `ahead` stages of the item's next flush: their operands wait in
      // shared memory, so the MMAs resume as soon as the accumulator is free.
      // They reuse buffers that this flush's MMAs release, so they never wait
      // on the epilogue (ahead <= NS).
      const int ahead = min(NS, FLUSH);
      int jdone = 0;  // stages of the item generated so far
      for (int j0 = 0; j0 < d.nst && ok; j0 += FLUSH) {
        const int j1 = min(d.nst, j0 + FLUSH);
        const int jend = min(d.nst, j1 + ahead);
        // this team's stages of [jdone, jend): global stages gs + (j - jdone)
        // with gs % nteams == team
        const uint32_t gs_end = gs + (uint32_t)(jend - jdone);
        for (; my_gs < gs_end && ok && generates;
             my_gs += (uint32_t)nteams, ring.advance((uint32_t)nteams, (uint32_t)NS)) {
          const int s = (int)ring.s;
          const uint32_t par = ring.ph;
          const int rs = (int)(my_gs & (TC_NREC - 1));
          // A parity wait is exact only while the barrier's previous phase
          // has completed.  For the stage barrier that holds because this
          // team's previous stage passed it (teams <= stages).  For the
          // record barrier it follows from this order: once stage gs is free
          // the MMAs have consumed stage gs - NS, so the records of every
          // stage up to gs - NS, gs - NREC among them (NREC >= NS), have
          // landed -- even when a record copy is withheld (fault injection).
          if (!wait_warp<kCluster>(smem_empty(s), par ^ 1, abort_flag, p.err, p.wait_ns)) { ok = false; break; }
          if (!wait_warp(rec_full(rs), (my_gs / TC_NREC) & 1, abort_flag, p.err, p.wait_ns)) { ok = false; break; }
          const SrcRec32* recs = reinterpret_cast<const SrcRec32*>(rec_smem + (size_t)rs * REC);
          const uint32_t stage_op = op_base + (uint32_t)s * stage_bytes;
          // unit u (sources 8 u .. 8 u + 7 of the stage) of slot index i
          auto unit = [&](int i, int u) {
            const uint32_t tile = stage_op + (uint32_t)u_slot[i] * TC_SLOT + rowoff;
            if constexpr (kForm == 0) {
              uint4 re_h = make_uint4(0, 0, 0, 0), im_h = re_h, re_l = re_h, im_l = re_h;
              if (u_ok[i]) {
                float rv[8], iv[8];
                gen_unit(recs + u * 8, i == 0 ? uc0 : Us[u_a[i]], beam + u_a[i], Np, dx, dy,
                         dlim, 1.f, rv, iv);
                split_pack(rv, re_h, re_l);
                split_pack(iv, im_h, im_l);
              }
              sts128(tile + ((uint32_t)(u ^ r8) << 4), re_h);
              sts128(tile + ((uint32_t)((2 + u) ^ r8) << 4), im_h);
              sts128(tile + ((uint32_t)((4 + u) ^ r8) << 4), re_l);
              sts128(tile + ((uint32_t)((6 + u) ^ r8) << 4), im_l);
            } else {
              uint4 re_h = make_uint4(0, 0, 0, 0), im_h = re_h;
              uint2 re_x = make_uint2(0, 0), im_x = re_x, re_l = re_x, im_l = re_x;
              if (u_ok[i]) {
                float rv[8], iv[8];
                gen_unit(recs + u * 8, i == 0 ? uc0 : Us[u_a[i]], beam + u_a[i], Np, dx, dy,
                         dlim, csc, rv, iv);
                split_f16_e4m3(rv, re_h, re_x, re_l);
                split_f16_e4m3(iv, im_h, im_x, im_l);
              }
              sts128(tile + ((uint32_t)(u ^ r8) << 4), re_h);
              sts128(tile + ((uint32_t)((4 + u) ^ r8) << 4), im_h);
              const uint32_t t8 = tile + tile8_off + (uint32_t)(u & 1) * 8u;
              const int c8 = u >> 1;
              sts64(t8 + ((uint32_t)(c8 ^ r8) << 4), re_x);
              sts64(t8 + ((uint32_t)((2 + c8) ^ r8) << 4), im_x);
              sts64(t8 + ((uint32_t)((4 + c8) ^ r8) << 4), re_l);
              sts64(t8 + ((uint32_t)((6 + c8) ^ r8) << 4), im_l);
            }
          };
          // one copy of the unit code (a second unrolled copy costs more in
          // instruction-cache misses than its static indices save)
#pragma unroll 1
          for (int k = 0; k < UPT; ++k) {
            const int u = sg * UPT + k;
            if (kCluster) {
              // static unit indices keep the unit tables in registers (a CTA
              // that generates owns at least one slot)
              unit(0, u);
              if (nfill > 1) unit(1, u);
              if (nfill > 2) unit(2, u);
            } else {
#pragma unroll
              for (int i = 0; i < 3; ++i)
                if (i < nfill) unit(i, u);
            }
          }
          // operands of this stage written: one arrival per warp (each lane
          // fences its own writes for the tensor core and the copy engine)
          fence_async_smem();
          __syncwarp();
          if (lane == 0) {
            mbar_arrive(smem_full(s));
            if (kCluster) mbar_arrive(gen_done(s));
            mbar_arrive(rec_empty(rs));  // the records may be reloaded
          }
        }
        gs = gs_end;
        if (!ok) break;
        jdone = jend;
        // ------------------------------------------------------- epilogue --
        // the sum of stages [j0, j1): stored into the partial for the first
        // flush of the item, added to it (at L2, no load) for the later ones;
        // the FP16 + FP8 form takes its slice scale out (exact)
        const bool first = j0 == 0;
        if (!wait_warp(acc_full, ic & 1, abort_flag, p.err, p.wait_ns)) { ok = false; break; }
        tc_fence_after();
        // a warp reads its lane quadrant q of TMEM; its 128-column blocks cb
        // (pair cb & 1, plane cb >> 1: Re, Im) are every (generator warps /
        // 4)-th from warp / 4
#pragma unroll 1
        for (int cb = warp >> 2; cb < 4; cb += TC_GEN_WARPS / 4) {
          const int q = warp & 3;
          const int pr = cb & 1, plane = cb >> 1;
          if (pr < g_npairs) {
            const int I = __ldg(&gp->pI[pr]), J = __ldg(&gp->pJ[pr]);
            float* out = SIM_P(d, partial) +
                         (((size_t)d.sl * SIM_I(d, nchunk) + d.k) * 2 + plane) * (size_t)Np * Np;
            const int a = I * TC_ROWS + q * 32 + lane;
            if (I <= J) {
              // partial[b][a] = V[a][b], a contiguous across the warp
#pragma unroll 1
              for (int c32 = 0; c32 < 4; ++c32) {
                float v[32];
                tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(cb * 128 + c32 * 32), v);
                if (kForm == 1) {
#pragma unroll
                  for (int c = 0; c < 32; ++c) v[c] *= inv_c2;
                }
                const int b0 = J * TC_ROWS + c32 * 32;
                if (first) {
#pragma unroll
                  for (int c = 0; c < 32; ++c) out[(size_t)(b0 + c) * Np + a] = v[c];
                } else {
#pragma unroll
                  for (int c = 0; c < 32; ++c) red_add(out + (size_t)(b0 + c) * Np + a, v[c]);
                }
              }
            } else {
              // below the diagonal (a > b): partial[a][b] = V[b][a] = conj V[a][b],
              // 32 consecutive b per lane
              const float sg_ = (plane ? -1.f : 1.f) * inv_c2;
#pragma unroll 1
              for (int c32 = 0; c32 < 4; ++c32) {
                float v[32];
                tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(cb * 128 + c32 * 32), v);
                float4* o4 = reinterpret_cast<float4*>(out + (size_t)a * Np + J * TC_ROWS + c32 * 32);
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                  const float4 x = make_float4(sg_ * v[4 * c], sg_ * v[4 * c + 1],
                                               sg_ * v[4 * c + 2], sg_ * v[4 * c + 3]);
                  if (first) o4[c] = x;
                  else red_add4(o4 + c, x);
                }
              }
            }
          }
        }
        tc_fence_before();
        mbar_arrive(acc_empty);
        ++ic;
      }  // flushes of the item
      if (!ok) break;
    }
  } else if (warp == TC_PRODUCER_WARP) {
    // ----------------------------------------------------- TMA producer --
    // The claiming thread (this CTA's producer; in cluster mode rank 0's)
    // takes the next item when it is about to load its records, so an item
    // is held by a CTA only once that CTA is ready for it.
    const bool claimer = rank == 0;
    if (lane == 0 && (generates || claimer)) {
      uint32_t gs = 0;
      ItemInfo d;
      bool ok = true;
      for (uint32_t k = 0; ok; ++k) {
        long long it;
        if (claimer) {
          const int slot = (int)(k % TC_ITEM_RING);
          // every reader of every CTA has read the slot's previous item
          if (!wait1<kCluster>(item_empty(slot), ((k / TC_ITEM_RING) & 1) ^ 1, abort_flag, p.err,
                               p.wait_ns)) { ok = false; break; }
          it = claim_item(p);
          if (kCluster) {
            for (int r = 0; r < csize; ++r) {
              st_cluster_b64(map_to_rank(smem_u32(item_ring + slot), (uint32_t)r), it);
              mbar_arrive_cluster(map_to_rank(item_full(slot), (uint32_t)r));
            }
          } else {
            item_ring[slot] = it;
            mbar_arrive(item_full(slot));  // release: the index is visible first
          }
        } else if (!read_item(k, it, one_thread{})) {
          ok = false;
          break;
        }
        if (it < 0) break;
        if (!generates) continue;
        if (!decode_item<kCluster, kTable, KS>(p, it, rank, d)) continue;
        for (int j = 0; j < d.nst; ++j, ++gs) {
          const int r = (int)(gs & (TC_NREC - 1));
          const uint32_t par = (gs / TC_NREC) & 1;
          // this CTA's generators have finished reading the previous round
          if (!wait1(rec_empty(r), par ^ 1, abort_flag, p.err, p.wait_ns)) { ok = false; break; }
          // fault injection: stage 0 never fills, so its consumers time out
          if (p.stall && gs == 0) continue;
          mbar_expect_tx(rec_full(r), REC);
          tma_load_2d(rec_base + (uint32_t)r * REC, &rec_map, rec_full(r), 0,
                      SIM_I(d, rec_row0) + d.tl * SIM_I(d, rec_stride) + d.s0 + j * KS);
        }
      }
      // let the copies still in flight land before the CTA can exit
      const uint32_t first = gs > (uint32_t)TC_NREC ? gs - TC_NREC : 0;
      for (uint32_t g = first; g < gs; ++g)
        wait_drain(rec_full((int)(g & (TC_NREC - 1))), (g / TC_NREC) & 1, p.err, p.wait_ns);
    }
  } else if (warp == TC_MMA_WARP) {
    // ------------------------------------------------------- MMA issuer --
    if (lane == 0) {
      uint32_t ic = 0;
      StageRing ring;  // operand stage of the next MMA
      ItemInfo d;
      bool ok = true;
      const uint16_t cmask = kCluster ? (uint16_t)__ldg(&mine->commit_mask) : (uint16_t)1;
      for (uint32_t k = 0; ok; ++k) {
        long long it;
        if (!read_item(k, it, one_thread{}) || it < 0) break;
        if (!decode_item<kCluster, kTable, KS>(p, it, rank, d)) continue;
        const TcGroup* gp = SIM_P(d, groups) + d.g;
        const int nm = __ldg(&gp->n_mma);
        const uint32_t abt = kForm == 0 ? 1u : 0u;  // BF16, or FP16 / E4M3
        const uint32_t idp = idesc_mma(nm, false, abt), idn = idesc_mma(nm, true, abt);
        const uint32_t a0 = desc_lo(op_base + (uint32_t)__ldg(&gp->sa) * TC_SLOT);
        const uint32_t b0 = desc_lo(op_base);
        for (int j0 = 0; j0 < d.nst && ok; j0 += FLUSH) {
          const int j1 = min(d.nst, j0 + FLUSH);
          // the generators have read the accumulator of the last flush
          if (!wait1(acc_empty, (ic & 1) ^ 1, abort_flag, p.err, p.wait_ns)) { ok = false; break; }
          tc_fence_after();
          for (int j = j0; j < j1; ++j, ring.advance(1u, (uint32_t)NS)) {
            const int s = (int)ring.s;
            const uint32_t par = ring.ph;
            if (!wait1(smem_full(s), par, abort_flag, p.err, p.wait_ns)) { ok = false; break; }
            // arm the next round of this stage for the peers' pushes (they can
            // only come after this round's MMAs release the slot)
            if (recv_bytes) mbar_expect_tx(smem_full(s), recv_bytes);
            tc_fence_after();
            const uint32_t so = ((uint32_t)s * stage_bytes) >> 4;
            if constexpr (kForm == 0) {
              issue_group(tmem, a0 + so, b0 + so, idp, idn, j == j0);
            } else {
              const uint32_t o8 = tile8_off >> 4;
              issue_group_f16f8(tmem, a0 + so, b0 + so, a0 + so + o8, b0 + so + o8, idp, idn,
                                j == j0);
            }
            // the stage's slots may be refilled -- here and, in cluster mode,
            // by the CTAs that wrote them -- once these MMAs have read them
            if (kCluster && cmask != (uint16_t)(1u << rank)) mma_commit_multicast(smem_empty(s), cmask);
            else mma_commit(smem_empty(s));
          }
          if (!ok) break;
          mma_commit(acc_full);
          ++ic;
        }  // flushes of the item
      }
      // every MMA issued by this thread completes before TMEM is released
      mma_commit(drain);
      wait_drain(drain, 0, p.err, p.wait_ns);
    }
  }

  if (kCluster && warp == TC_PUSH_WARP && lane == 0 && nown > 0) {
    // ---------------------------------------------- DSMEM tile pusher --
    StageRing ring;  // operand stage of the next push
    ItemInfo d;
    bool ok = true;
    for (uint32_t k = 0; ok; ++k) {
      long long it;
      if (!read_item(k, it, one_thread{}) || it < 0) break;
      if (!decode_item<kCluster, kTable, KS>(p, it, rank, d)) continue;
      for (int j = 0; j < d.nst; ++j, ring.advance(1u, (uint32_t)NS)) {
        const int s = (int)ring.s;
        const uint32_t par = ring.ph;
        if (!wait1(gen_done(s), par, abort_flag, p.err, p.wait_ns)) { ok = false; break; }
        const uint32_t stage_op = op_base + (uint32_t)s * stage_bytes;
        for (int k = 0; k < nown; ++k) {
          const uint32_t src = stage_op + (uint32_t)__ldg(&mine->own_slot[k]) * TC_SLOT;
          const int nd = __ldg(&mine->ndst[k]);
          for (int q = 0; q < nd; ++q) {
            const uint32_t rr = (uint32_t)__ldg(&mine->dst_rank[k][q]);
            const uint32_t dst = stage_op + (uint32_t)__ldg(&mine->dst_slot[k][q]) * TC_SLOT;
#pragma unroll
            for (int x = 0; x < TILES; ++x)
              bulk_push(map_to_rank(dst + x * tile8_off, rr), src + x * tile8_off, TC_SLOT,
                        map_to_rank(smem_full(s), rr));
          }
        }
      }
    }
    bulk_wait_all();
  }

  tc_fence_before();
  __syncthreads();
  // no CTA leaves while a peer may still write to its shared memory
  if (kCluster) cluster_sync_all();
  if (warp == TC_MMA_WARP) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TC_TMEM_COLS)
                 : "memory");
  }
}

#undef SIM_I
#undef SIM_P

// ------------------------------------------------------------------- host --
namespace {

std::vector<TcGroup> make_groups(int nant) {
  const int nb = ceil_div(nant, TC_ROWS);
  auto rows_of = [&](int blk) { return std::min(TC_ROWS, nant - blk * TC_ROWS); };
  auto ncols = [&](int blk) { return ((rows_of(blk) + 15) / 16) * 16; };
  // (row block, column block) pairs of each group; the column blocks of a
  // group are different and only the last may be partly valid
  std::vector<std::vector<std::pair<int, int>>> raw;
  std::vector<int> singles;  // rows whose last pair (I, nb - 1) is left over
  for (int I = 0; I < nb; ++I) {
    int J = I;
    for (; J + 1 < nb; J += 2) raw.push_back({{I, J}, {I, J + 1}});
    if (J < nb) singles.push_back(I);
  }
  // the left-over pairs all end on block nb - 1: taken as (nb - 1, I) they
  // share the row block, two per group (ascending I, so the diagonal pair
  // (nb - 1, nb - 1), whose block may be partial, comes last)
  for (size_t k = 0; k < singles.size(); k += 2) {
    std::vector<std::pair<int, int>> g{{nb - 1, singles[k]}};
    if (k + 1 < singles.size()) g.push_back({nb - 1, singles[k + 1]});
    raw.push_back(g);
  }
  std::vector<TcGroup> out;
  for (auto& prs : raw) {
    TcGroup g{};
    g.npairs = (int)prs.size();
    g.nslots = 0;
    auto slot_of = [&](int blk) {
      for (int s = 0; s < g.nslots; ++s)
        if (g.slot_block[s] == blk) return s;
      g.slot_block[g.nslots] = blk;
      g.slot_rows[g.nslots] = rows_of(blk);
      return g.nslots++;
    };
    // column blocks first (slots 0 and 1, side by side), then the row block
    for (int q = 0; q < g.npairs; ++q) {
      g.pI[q] = prs[q].first;
      g.pJ[q] = prs[q].second;
      g.pN[q] = ncols(prs[q].second);
      slot_of(prs[q].second);
    }
    g.sa = slot_of(prs[0].first);
    g.n_mma = g.npairs == 2 ? TC_ROWS + g.pN[1] : g.pN[0];
    out.push_back(g);
  }
  return out;
}

// Cluster mode: each block is generated by one CTA of the cluster (among
// the groups that use it, the one with the fewest generated rows so far) and
// sent to the others; fills the sharing fields of every group.
void plan_cluster(std::vector<TcGroup>& gs, int nant) {
  const int C = (int)gs.size();
  const int nb = ceil_div(nant, TC_ROWS);
  std::vector<int> load(C, 0);
  auto slot_in = [&](int g, int blk) {
    for (int s = 0; s < gs[g].nslots; ++s)
      if (gs[g].slot_block[s] == blk) return s;
    return -1;
  };
  for (auto& g : gs) {
    g.nown = 0;
    g.write_mask = 0;
  }
  for (int b = 0; b < nb; ++b) {
    int owner = -1;
    for (int g = 0; g < C; ++g)
      if (slot_in(g, b) >= 0 && (owner < 0 || load[g] < load[owner])) owner = g;
    if (owner < 0) continue;
    load[owner] += std::min(TC_ROWS, nant - b * TC_ROWS);
    TcGroup& o = gs[owner];
    const int k = o.nown++;
    o.own_slot[k] = slot_in(owner, b);
    o.ndst[k] = 0;
    o.write_mask |= 1 << owner;
    for (int g = 0; g < C; ++g) {
      if (g == owner || slot_in(g, b) < 0) continue;
      o.dst_rank[k][o.ndst[k]] = g;
      o.dst_slot[k][o.ndst[k]] = slot_in(g, b);
      ++o.ndst[k];
      o.write_mask |= 1 << g;
    }
  }
  for (int x = 0; x < C; ++x) {
    int writers = 0, commit = 1 << x, targets = 0;
    for (int o = 0; o < C; ++o) {
      if ((gs[o].write_mask >> x) & 1) {
        ++writers;
        commit |= 1 << o;
      }
      if (o != x && ((gs[x].write_mask >> o) & 1)) ++targets;
    }
    // local generator warps (if this CTA generates) + the MMA thread's arming
    // of the bytes pushed by peers
    int recv = 0;
    for (int o = 0; o < C; ++o)
      if (o != x)
        for (int k = 0; k < gs[o].nown; ++k)
          for (int q = 0; q < gs[o].ndst[k]; ++q)
            if (gs[o].dst_rank[k][q] == x) ++recv;
    gs[x].recv_slots = recv;
    (void)writers;
    gs[x].commit_mask = commit;
    gs[x].empty_count = 1 + targets;
  }
}

bool use_cluster(int ngroups) { return ngroups > 1 && ngroups <= TC_MAX_CLUSTER; }

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
  }
  return fn;
}

}  // namespace

int tc_num_groups(int nant) { return (int)make_groups(nant).size(); }

namespace {
template <int kForm>
int team_warps_for(int nant) {
  constexpr int T = TcLayout<kForm>::TEAM;
  return nant <= 32 ? T / 4 : nant <= 64 ? T / 2 : T;
}
}  // namespace

int tc_team_warps(int nant) { return team_warps_for<0>(nant); }

size_t tc_group_table_bytes(int nant) { return sizeof(TcGroup) * make_groups(nant).size(); }

int tc_fill_group_table(int nant, void* host_buf) {
  auto g = make_groups(nant);
  if (use_cluster((int)g.size())) plan_cluster(g, nant);
  std::copy(g.begin(), g.end(), static_cast<TcGroup*>(host_buf));
  return (int)g.size();
}

int tc_chunk_sources(int nsrc, int nslices, int ngroups, int num_sms) {
  // about 40 items per cluster (or per CTA without clusters), so that the
  // run-time claiming leaves a short tail, in chunks of 1k-32k sources
  // (about half the catalogue is above the horizon)
  const long long nchunk =
      std::max<long long>(1, (40LL * num_sms + (long long)nslices * ngroups - 1) /
                                 ((long long)nslices * ngroups));
  const long long up = std::max(nsrc / 2, 1);
  long long c = (up + nchunk - 1) / nchunk;
  c = std::min<long long>(32768, std::max<long long>(1024, c));
  c = (c + 31) / 32 * 32;
  return (int)c;
}

size_t tc_sim_table_bytes(int nsims) { return sizeof(TcSim) * (size_t)std::max(nsims, 1); }

cudaError_t tc_configure() {
  static bool done = false;
  if (done) return cudaSuccess;
  for (const void* k : {reinterpret_cast<const void*>(tc_vis_kernel<false, false, 0>),
                        reinterpret_cast<const void*>(tc_vis_kernel<false, true, 0>),
                        reinterpret_cast<const void*>(tc_vis_kernel<true, false, 0>),
                        reinterpret_cast<const void*>(tc_vis_kernel<true, true, 0>),
                        reinterpret_cast<const void*>(tc_vis_kernel<false, false, 1>),
                        reinterpret_cast<const void*>(tc_vis_kernel<false, true, 1>),
                        reinterpret_cast<const void*>(tc_vis_kernel<true, false, 1>),
                        reinterpret_cast<const void*>(tc_vis_kernel<true, true, 1>)}) {
    const cudaError_t e =
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM_LIMIT);
    if (e != cudaSuccess) return e;
  }
  done = true;
  return cudaSuccess;
}

namespace {

// The launches of one fused-kernel call in form kForm (see launch_tc_batch).
template <int kForm>
cudaError_t launch_form(const TcSimDesc* sims, int nsims, const void* rec, long long rec_rows,
                        void* d_table, void* h_table, int* err, unsigned long long* claim,
                        int num_sms, cudaStream_t st, unsigned long long wait_ns, int stall,
                        TcShare* share) {
  constexpr int KS = TcForm<kForm>::KS;
  constexpr int TILES = TcForm<kForm>::TILES;
  constexpr int TC_GEN_WARPS = TcLayout<kForm>::GEN_WARPS;
  constexpr int TC_TEAM_WARPS = TcLayout<kForm>::TEAM;
  constexpr int TC_THREADS = tc_threads<kForm>();
  auto encode = encode_fn();
  if (!encode) return cudaErrorNotSupported;
  CUtensorMap map;
  const cuuint64_t gdim[2] = {8, (cuuint64_t)rec_rows};
  const cuuint64_t gstride[1] = {sizeof(SrcRec32)};
  const cuuint32_t box[2] = {8, (cuuint32_t)KS};
  const cuuint32_t estride[2] = {1, 1};
  CUresult r = encode(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(rec), gdim,
                      gstride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
                      CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;

  // cluster mode when every simulation has the same (clusterable) group layout
  bool cluster = use_cluster(sims[0].ngroups);
  int max_slots = 1, team_warps = 1;
  for (int i = 0; i < nsims; ++i) {
    if (sims[i].ngroups != sims[0].ngroups) cluster = false;
    max_slots = std::max(max_slots, sims[i].max_slots);
    team_warps = std::max(team_warps, team_warps_for<kForm>(sims[i].nant));
  }
  TcSim* tab = static_cast<TcSim*>(h_table);
  long long items = 0;
  for (int i = 0; i < nsims; ++i) {
    const TcSimDesc& L = sims[i];
    TcSim t{};
    t.counts = L.counts;
    t.U = static_cast<const Ucoef32*>(L.U);
    t.beamT = L.beamT;
    t.umax = L.umax;
    t.sbound = L.sbound;
    t.partial = L.partial;
    t.groups = static_cast<const TcGroup*>(L.groups);
    t.item0 = items;
    t.rec_row0 = (int)L.rec_row0;
    t.rec_stride = L.rec_stride;
    t.nt = L.nt;
    t.nf = L.nf;
    t.Np = L.Np;
    t.PP = L.P * L.P;
    t.dx = L.P > 1 ? 1 : 0;
    t.dy = L.P > 1 ? L.P : 0;
    t.chunk = L.chunk;
    t.nchunk = ceil_div(std::max(L.nsrc, 1), L.chunk);
    t.ngroups = L.ngroups;
    tab[i] = t;
    items += (long long)L.nt * L.nf * t.nchunk * (cluster ? 1 : L.ngroups);
  }
  if (items == 0) return cudaSuccess;
  const bool table = nsims > 1;
  cudaError_t e = cudaSuccess;
  if (table) {
    e = cudaMemcpyAsync(d_table, h_table, sizeof(TcSim) * nsims, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
  }

  // the claim counter starts at zero (in stream order, before the launches)
  e = cudaMemsetAsync(claim, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  TcParams p{};
  p.claim = claim;
  p.claim_mode = kClaimCount;
  p.sims = static_cast<const TcSim*>(d_table);
  p.one = tab[0];
  p.nsims = nsims;
  p.total_items = items;
  p.max_slots = max_slots;
  p.err = err;
  p.wait_ns = wait_ns ? wait_ns : TC_WAIT_NS;
  p.stall = stall;
  p.team_warps = team_warps;
  const int per_stage = TILES * p.max_slots * TC_SLOT;
  // records and the barrier block (barriers, item ring, TMEM holder: at most
  // 8 (2 NREC + 3 NS + 3 + 2 RING + RING) + 8 = 472 bytes)
  constexpr int TC_NREC = TcForm<kForm>::NREC;
  const int fixed = TC_NREC * KS * 32 + 480;
  const int max_stages = std::min(TC_MAX_STAGES, (TC_SMEM_LIMIT - fixed) / per_stage);
  p.nstages = max_stages;
  if (sims[0].tune.stages > 0) p.nstages = std::min(p.nstages, sims[0].tune.stages);
  // A team waits on a stage's barriers by phase parity, which tells apart
  // only consecutive phases: a team may run at most one round of a stage
  // ahead of the MMAs, which holds while the teams are no more than the
  // stages (each team's previous stage was released before it).  Small
  // teams of one-slot launches are widened, and a stage cap below the
  // number of teams raised, until that holds.
  while ((TC_GEN_WARPS / p.team_warps > p.nstages || TC_GEN_WARPS / p.team_warps > TC_NREC) &&
         p.team_warps < TC_TEAM_WARPS)
    p.team_warps *= 2;
  const int teams = std::max(TC_GEN_WARPS / p.team_warps, cluster ? TC_GEN_WARPS / TC_TEAM_WARPS : 1);
  p.nstages = std::min(max_stages, std::max(p.nstages, teams));
  if (p.nstages < 2 || teams > p.nstages || TC_GEN_WARPS / p.team_warps > TC_NREC ||
      p.nstages > TC_NREC)
    return cudaErrorInvalidConfiguration;
  const int smem = fixed + p.nstages * per_stage;
  e = tc_configure();
  if (e != cudaSuccess) return e;
  // The SM's on-chip memory is split between shared memory and the L1 cache
  // that serves the beam gathers in fixed sizes; ask for the smallest
  // shared size that holds the launch (with the CTA's reserved 1 KB), so
  // that the rest is L1.
  {
    int carve_kb = 228;
    for (int kb : {100, 132, 164, 196, 228})
      if (kb * 1024 >= smem + 1024) {
        carve_kb = kb;
        break;
      }
    const int pct = (carve_kb * 100 + 227) / 228;
    for (const void* k : {reinterpret_cast<const void*>(tc_vis_kernel<false, false, kForm>),
                          reinterpret_cast<const void*>(tc_vis_kernel<false, true, kForm>),
                          reinterpret_cast<const void*>(tc_vis_kernel<true, false, kForm>),
                          reinterpret_cast<const void*>(tc_vis_kernel<true, true, kForm>)}) {
      e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
      if (e != cudaSuccess) return e;
    }
  }
  if (!cluster) {
    const long long grid = std::min<long long>(num_sms, items);
    if (table) tc_vis_kernel<false, true, kForm><<<(int)grid, TC_THREADS, smem, st>>>(map, p);
    else tc_vis_kernel<false, false, kForm><<<(int)grid, TC_THREADS, smem, st>>>(map, p);
    return cudaGetLastError();
  }
  // cluster mode: one CTA per group, items are (slice, chunk)
  const int C = sims[0].ngroups;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(TC_THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cfg.gridDim = dim3((unsigned)(C * (num_sms / C)));
  // co-resident clusters for this cluster size and shared memory (cached:
  // the query is host-side and stays valid)
  static int cached_n[2][TC_MAX_CLUSTER + 1][TC_MAX_STAGES + 1] = {};
  int& nclusters = cached_n[table][C][p.nstages];
  if (nclusters == 0) {
    e = table ? cudaOccupancyMaxActiveClusters(&nclusters, tc_vis_kernel<true, true, kForm>,
                                               &cfg)
              : cudaOccupancyMaxActiveClusters(&nclusters,
                                               tc_vis_kernel<true, false, kForm>, &cfg);
    if (e != cudaSuccess) return e;
  }
  if (nclusters < 1) return cudaErrorInvalidConfiguration;
  const int ncl = (int)std::min<long long>(nclusters, items);
  cfg.gridDim = dim3((unsigned)(C * ncl));
  const int leftover = num_sms - C * ncl;
  if (share && !table && leftover >= 4) {
    // The SMs no cluster fits on run the same items, one CTA per group item,
    // in a second launch: the two claim from the two ends of one packed
    // counter (kClaimFront / kClaimBack), so each item is computed once and
    // the split adapts at run time (a one-CTA item, which generates all of
    // its group's blocks itself, runs at about 0.7 of a cluster CTA's rate).
    // The cluster launch goes to the higher-priority stream; should the
    // one-CTA launch take an SM a cluster needed first, that cluster claims
    // fewer items and nothing waits for it.
    if ((e = cudaEventRecord(share->fork, st)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(share->hi, share->fork, 0)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(share->lo, share->fork, 0)) != cudaSuccess) return e;
    p.claim_mode = kClaimFront;
    p.group_items = items * C;
    cfg.stream = share->hi;
    if ((e = cudaLaunchKernelEx(&cfg, tc_vis_kernel<true, false, kForm>, map, p)) !=
        cudaSuccess)
      return e;
    TcParams q = p;
    q.total_items = items * C;
    q.claim_mode = kClaimBack;
    tc_vis_kernel<false, false, kForm><<<leftover, TC_THREADS, smem, share->lo>>>(map, q);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaEventRecord(share->join_hi, share->hi)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(share->join_lo, share->lo)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(st, share->join_hi, 0)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(st, share->join_lo, 0)) != cudaSuccess) return e;
    share->launched = 2;
    return cudaSuccess;
  }
  e = table ? cudaLaunchKernelEx(&cfg, tc_vis_kernel<true, true, kForm>, map, p)
            : cudaLaunchKernelEx(&cfg, tc_vis_kernel<true, false, kForm>, map, p);
  if (e != cudaSuccess) return e;
  if (share) share->launched = 1;
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_tc_batch(const TcSimDesc* sims, int nsims, const void* rec, long long rec_rows,
                            void* d_table, void* h_table, int* err, unsigned long long* claim,
                            int num_sms, cudaStream_t st, unsigned long long wait_ns, int stall,
                            TcShare* share) {
  if (share) share->launched = 0;
  if (nsims <= 0 || rec_rows <= 0) return cudaSuccess;
  // one form per launch
  for (int i = 1; i < nsims; ++i)
    if (sims[i].form != sims[0].form) return cudaErrorInvalidValue;
  if (sims[0].form == 1) {
    for (int i = 0; i < nsims; ++i)
      if (!sims[i].sbound) return cudaErrorInvalidValue;
    return launch_form<1>(sims, nsims, rec, rec_rows, d_table, h_table, err, claim, num_sms, st,
                          wait_ns, stall, share);
  }
  if (sims[0].form != 0) return cudaErrorInvalidValue;
  return launch_form<0>(sims, nsims, rec, rec_rows, d_table, h_table, err, claim, num_sms, st,
                        wait_ns, stall, share);
}

size_t tc_partial_floats(int Np, int nsrc, int nslices, int chunk) {
  return (size_t)nslices * ceil_div(std::max(nsrc, 1), chunk) * 2 * (size_t)Np * Np;
}

int tc_max_slots(int nant) {
  int m = 1;
  for (auto& g : make_groups(nant)) m = std::max(m, g.nslots);
  return m;
}

}  // namespace hv
