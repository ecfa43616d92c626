// hv_kernels.h -- host-side launchers of the kernels of libheravis.so
// (internal to the library; the public C ABI is include/heravis.h).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace hv {

// --- batches: table-driven preparation and reduction -------------------------
// One simulation of a batch for the launches that prepare or reduce every
// simulation of the batch at once (device pointers; the batch's arena).
// Each such launch flattens the blocks (or elements) of all simulations into
// one index range; `pre` of that launch holds the nsims + 1 prefix sums, and
// a block finds its simulation by binary search.
struct PrepSim {
  const float* antpos;
  const float* eq2tops;
  const float* crd_eq;
  const float* I_sky;
  const float* bm;       // (F, nant, P, P)
  const double* freqs;   // (F,) device
  float* beamT;          // [F][P*P][Np]
  void* U;               // Ucoef32 [T][F][Np]
  float* umax;           // [T * F]
  int* counts;           // [T]
  int* blk;              // [T][prep_blocks(S)]
  unsigned long long* kv;  // sort_pad(S) words of the spatial sort (S > 0)
  float* crd_s;          // (3, S) in spatial order
  float* I_s;            // (S,) in spatial order
  void* rec;             // SrcRec32 rows of time 0 (rec_stride per time)
  float* partial;        // [T * F][nchunk][2][Np][Np]
  void* out;             // (F, T, nant, nant) complex64
  int nant, Np, T, F, S, P, rec_stride, chunk;
};
// Prefix sums of the flattened index range of each batch launch (nsims + 1
// entries each, device memory).
struct PrepPre {
  const long long* beam;   // transpose tiles (32 x 32) x frequencies
  const long long* ucoef;  // elements T * F * Np
  const long long* slice;  // slices T * F
  const long long* key;    // sort keys: sort_pad(S) per simulation with sources, else 0
  const long long* pair;   // compare-exchange pairs: key / 2
  const long long* tile;   // shared-memory sort tiles: key / 2048
  const long long* prep;   // prep blocks x times
  const long long* rel;    // units of 256 records x times (tc_relative)
  const long long* red;    // upper 32 x 32 output tiles x slices
};
struct PrepTotals {
  long long beam, ucoef, slice, key, pair, tile, prep, rel, red;
  int max_key;             // the largest sort_pad(S) of the batch (0: no sources)
};
// The preparation of every simulation of a batch (spatial sort, beam
// layout, phase coefficients and their bounds, records), table-driven: the
// number of launches depends on the largest simulation's source count, not
// on the number of simulations.  *launches is set to the kernels launched.
cudaError_t launch_prepare_batch(const PrepSim* sims, int nsims, const PrepPre& pre,
                                 const PrepTotals& tot, int* launches, cudaStream_t st);
// The spatial sort of every simulation of a batch (hv_sort.cu): each one's
// keys are sorted within its own segment, exactly as launch_sort_sources
// sorts them alone.
cudaError_t launch_sort_batch(const PrepSim* sims, int nsims, const PrepPre& pre,
                              const PrepTotals& tot, int* launches, cudaStream_t st);
// The split-K reduction of every simulation of a batch into its output.
cudaError_t launch_reduce_batch(const PrepSim* sims, int nsims, const PrepPre& pre,
                                const PrepTotals& tot, cudaStream_t st);

// --- hv_prep.cu ------------------------------------------------------------
// bm (nfreq, nant, P, P) -> beamT (nfreq, P*P, Np), zero for padded antennas.
template <typename R>
cudaError_t launch_beam_transpose(const R* bm, int nfreq, int nant, int P, int Np,
                                  R* beamT, cudaStream_t st);

// Phase coefficients for times [t0, t0 + nt) and every frequency:
// U[(tt * nfreq + f) * Np + a].
template <typename R>
cudaError_t launch_ucoef(const R* antpos, int nant, int Np, const R* eq2tops, int t0,
                         int nt, const double* d_freqs, int nfreq, void* U,
                         cudaStream_t st);

// Number of prep blocks for nsrc sources.
int prep_blocks(int nsrc);

// Horizon cut + beam corner for times [t0, t0 + nt): records of the sources
// with z > 0, in input order, into rec + tt * nsrc; counts into count[tt].
// block_counts needs prep_blocks(nsrc) * nt ints.
template <typename R>
cudaError_t launch_prep(const R* crd_eq, const R* I_sky, int nsrc, const R* eq2tops,
                        int t0, int nt, int P, int* block_counts, void* rec,
                        int* count, cudaStream_t st);

// Bound max_a (|U_x| + |U_y| + |U_z|) of every (time, frequency) slice of U
// (nslices x Np Ucoef32) into umax[nslices] (used by the fused kernel to
// decide when a phase may be taken relative to a nearby source).
cudaError_t launch_ubound(const void* U, int nslices, int Np, float* umax, cudaStream_t st);

// --- hv_sort.cu ------------------------------------------------------------
// Spatial (Morton) order of the sources: kv_buf needs sort_pad(nsrc) 64-bit
// words; writes the permuted crd_eq (3 x nsrc) and I_sky.  *launches is set
// to the number of kernels launched.
int sort_pad(int nsrc);
cudaError_t launch_sort_sources(const float* crd_eq, const float* I_sky, int nsrc, void* kv_buf,
                                float* crd_sorted, float* I_sorted, int* launches,
                                cudaStream_t st);

// launch_prep with records of time tt at rec + tt * rec_stride.
template <typename R>
cudaError_t launch_prep_strided(const R* crd_eq, const R* I_sky, int nsrc, const R* eq2tops,
                                int t0, int nt, int P, int* block_counts, void* rec,
                                size_t rec_stride, int* count, cudaStream_t st);

// Fused-path record preparation (hv_prep.cu): per-unit spread of directions
// in the pad word of each unit's first record, zero padding to a multiple of
// 32 (rec_stride >= round_up(nsrc, 32)).
cudaError_t launch_tc_relative(void* rec, size_t rec_stride, const int* counts, int nt, int nsrc,
                               cudaStream_t st);

// FP16 + FP8 form: pixmax[f][pix] = max over antennas of |beamT[f][pix][a]|
// (nfreq * P * P floats).
cudaError_t launch_beam_pixmax(const float* beamT, int nfreq, int P, int Np, float* pixmax,
                               cudaStream_t st);
// FP16 + FP8 form: sbound[tt * nf + f] (zeroed here) = a bound of |A| sqrt(I)
// over the records of time tt at frequency f, for the nt times of rec.
cudaError_t launch_slice_bound(const void* rec, size_t rec_stride, const int* counts, int nt,
                               int nsrc, const float* pixmax, int nf, int P, float* sbound,
                               cudaStream_t st);

// --- hv_plain.cu -----------------------------------------------------------
// Source chunk of the split-K sum over sources (plain path).
constexpr int kPlainChunk = 4096;

// v[s][a] (complex, Np per source) for the count[0] records of one slice.
template <typename R>
cudaError_t launch_gen_phasors(const void* rec, const int* count, int nsrc_max,
                               const void* U, const R* beamT, int Np, int nant, int P,
                               void* v, cudaStream_t st);

// Upper-triangle SIMT Hermitian product of v into partial sums, one chunk of
// kPlainChunk sources per grid row.
template <typename R>
cudaError_t launch_herk_plain(const void* v, const int* count, int nsrc_max, int Np,
                              R* partial, cudaStream_t st);

// For each of nt * nf slices (slice = tl * nf + f, partial sums at
// partial + slice * slice_stride, source count counts[tl]): sum the valid
// chunks (ceil(count / chunk) of them) in order and write the full Hermitian
// matrix (nant x nant complex R, row-major) to
// out + ((f * ntimes_out) + t0 + tl) * nant * nant.
template <typename R>
cudaError_t launch_reduce(const R* partial, size_t slice_stride, const int* counts, int nt,
                          int nf, int t0, int ntimes_out, int chunk, int Np, int nant, void* out,
                          cudaStream_t st);

// --- hv_tc.cu --------------------------------------------------------------
// Launch shape of the fused kernel; 0 everywhere = the defaults.
struct TcTune {
  int stages;  // cap on the operand stages in shared memory (>= the generator teams)
};
// One simulation of a fused-kernel launch (device pointers).
struct TcSimDesc {
  const int* counts;    // [nt] sources above the horizon per time
  const void* U;        // Ucoef32 [nt][nf][Np]
  const float* beamT;   // [nf][P*P][Np]
  const float* umax;    // [nt * nf] bound of |U|_1 per slice (launch_ubound)
  const float* sbound;  // [nt * nf] bound of |A| sqrt(I) per slice (form 1; launch_slice_bound)
  float* partial;       // [nt * nf][ceil(nsrc / chunk)][2][Np][Np]
  const void* groups;   // device group table (tc_fill_group_table for this nant)
  int ngroups, max_slots;
  long long rec_row0;   // first record row of time 0 in the launch's record tensor
  int rec_stride;       // records per time, a multiple of 32 >= nsrc
  int nt, nf, Np, nant, P, nsrc;
  int chunk;            // sources per split-K chunk (multiple of 32)
  int form;             // 0: split BF16; 1: FP16 + FP8 (needs sbound)
  TcTune tune;          // launch shape (the first simulation's applies to a launch)
};
size_t tc_sim_table_bytes(int nsims);
int tc_num_groups(int nant);
// Generator warps per stage of the fused kernel for nant antennas (launches
// whose simulations differ use the largest).
int tc_team_warps(int nant);
// One-time launch attributes of the fused kernel (call outside stream capture).
cudaError_t tc_configure();
// All items of nsims simulations in one persistent launch; its CTAs claim
// the items at run time from *claim (8 bytes of device memory that no other
// launch uses at the same time; zeroed here, in stream order).  rec: SrcRec32
// rows (rewritten by launch_tc_relative) of every simulation, rec_rows in
// all.  d_table / h_table: device and host (kept alive until the copy ran)
// buffers of tc_sim_table_bytes(nsims).  Cluster mode is used when every
// simulation has the same clusterable group layout.  wait_ns: limit of
// each device-side wait (0: 10 s); stall: fault injection (the first record
// copy is never issued, so the launch ends with a timeout status).
// share (one simulation in cluster mode): the SMs no cluster fits on run a
// share of the items in a second, concurrent launch (forked from st onto
// share->hi / share->lo and joined back); share->launched counts kernels.
struct TcShare {
  cudaStream_t hi, lo;                  // highest- and lowest-priority streams
  cudaEvent_t fork, join_hi, join_lo;   // timing disabled
  int launched;
};
cudaError_t launch_tc_batch(const TcSimDesc* sims, int nsims, const void* rec, long long rec_rows,
                            void* d_table, void* h_table, int* err, unsigned long long* claim,
                            int num_sms, cudaStream_t st, unsigned long long wait_ns = 0,
                            int stall = 0, TcShare* share = nullptr);
size_t tc_partial_floats(int Np, int nsrc, int nslices, int chunk);
int tc_chunk_sources(int nsrc, int nslices, int ngroups, int num_sms);
size_t tc_group_table_bytes(int nant);
int tc_fill_group_table(int nant, void* host_buf);
int tc_max_slots(int nant);

}  // namespace hv

// Context internals shared by the library's translation units (hv_api.cu).
struct hv_context;
cudaStream_t hv_context_stream(hv_context* ctx);
void hv_context_set_error(hv_context* ctx, const char* msg);
void hv_context_add_launches(hv_context* ctx, uint64_t n);
int hv_context_num_sms(hv_context* ctx);
// Page-locked host block of at least `bytes` (its size in *cap) from the
// context's pool of returned blocks, or newly allocated; nullptr on failure.
void* hv_context_host_take(hv_context* ctx, size_t bytes, size_t* cap);
// Returns a block to the pool (no copy may still read it).
void hv_context_host_give(hv_context* ctx, void* p, size_t cap);
// Profiling: the context owns and times the pair of recorded events.
bool hv_context_profiling(hv_context* ctx);
void hv_context_record_kernel(hv_context* ctx, cudaEvent_t e0, cudaEvent_t e1);
// Wait limit and fault injection of the fused kernel (hv_set_wait_limit).
uint64_t hv_context_wait_ns(hv_context* ctx);
// Streams and scratch of the context for shared fused launches (TcShare).
hv::TcShare* hv_context_share(hv_context* ctx);
int hv_context_stall(hv_context* ctx);
