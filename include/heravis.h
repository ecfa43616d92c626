/*
 * heravis.h -- C ABI of the GB300 visibility simulator (libheravis.so).
 *
 * The library is a drop-in for the one hot path of hera_gpu,
 * hera_gpu.vis.vis_gpu (reference hera_gpu/vis.py:144-262): per time, rotate
 * sources to topocentric, drop those below the horizon, bilinearly
 * interpolate each antenna's beam, form v[a,s] = A_a(l,m) sqrt(I_s)
 * exp(2 pi i nu tau_as) and return V[a,b] = sum_s v[a,s] conj(v[b,s]) as the
 * full Hermitian (ntimes, nant, nant) matrix.
 *
 * The reference exposes that path as a Python function only; these entry
 * points are what a foreign-function binding of it binds (the ctypes binding
 * shipped in hera_gpu_gb300/_native.py is one).
 *
 * Conventions
 *  - Every call returns an hv_status; hv_last_error() gives the message of the
 *    last failure on that context.  Bad shapes or arguments return
 *    HV_ERR_ARG (the reference raises AssertionError, vis.py:147,161-169).
 *  - precision 1: float32 inputs, complex64 output (interleaved re, im);
 *    precision 2: float64 inputs, complex128 output (vis.py:147-157).
 *  - Array layouts are C order, exactly as the reference's arguments:
 *      antpos  (nant, 3)            metres
 *      eq2tops (ntimes, 3, 3)       equatorial -> topocentric rotations
 *      crd_eq  (3, nsrc)            equatorial unit vectors
 *      I_sky   (nsrc,)              intensities (sqrt taken internally)
 *      bm_cube (nant, P, P)         beam on the grid linspace(-1,1,P),
 *                                   axis order [ant, y(m), x(l)]
 *      vis     (ntimes, nant, nant) output
 *    Multi-frequency calls take bm_cubes (nfreq, nant, P, P) and write
 *    vis (nfreq, ntimes, nant, nant).
 *  - Limits (HV_ERR_ARG beyond them): 1 <= nant <= 65536, 1 <= P <= 4096,
 *    ntimes x nfreq <= 2^31 - 1.
 *  - A context owns one CUDA stream and a workspace on one device; it is not
 *    thread-safe (one thread per context, or a lock around it).
 */
#ifndef HERAVIS_H
#define HERAVIS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  HV_OK = 0,
  HV_ERR_ARG = 1,         /* bad shape / argument (reference: AssertionError) */
  HV_ERR_OOM = 2,         /* device allocation failed or HBM budget exceeded  */
  HV_ERR_CUDA = 3,        /* CUDA runtime error                               */
  HV_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up               */
  HV_ERR_UNSUPPORTED = 5  /* no suitable GPU / method unavailable             */
} hv_status;

typedef enum {
  HV_METHOD_AUTO = 0,     /* tensor-core form for precision 1, FP64 for 2      */
  HV_METHOD_PLAIN = 1,    /* the reference's method: phasors to HBM, then an
                             FP32 (precision 1) / FP64 (precision 2) SIMT
                             Hermitian product                                 */
  HV_METHOD_TC_BF16 = 2,  /* fused: phasors generated in shared memory, split
                             BF16 tcgen05 products, FP32 accumulation in TMEM  */
  HV_METHOD_TC_FP16 = 3   /* fused, FP16 hi products and E4M3 (FP8) cross
                             terms of a per-(time, frequency) power-of-two
                             scaled split, FP32 accumulation in TMEM: about
                             2/3 of the tensor-core time of TC_BF16          */
} hv_method;

typedef struct hv_context hv_context;

/* Library version (major*10000 + minor*100 + patch). */
int hv_version(void);

/* Open a context on CUDA device `device`; `hbm_budget_bytes` caps the
 * workspace the context may hold (0 = no cap).  Replaces the import-time
 * pycuda.autoinit context of the reference (vis.py:1). */
int hv_create(hv_context** ctx, int device, size_t hbm_budget_bytes);
int hv_destroy(hv_context* ctx);
const char* hv_last_error(const hv_context* ctx);

/* Kernel launches issued by this context since creation (all methods). */
uint64_t hv_launch_count(const hv_context* ctx);

/* Drop-in for vis_gpu(antpos, freq, eq2tops, crd_eq, I_sky, bm_cube,
 * precision=...) (reference hera_gpu/vis.py:144-146).  Host buffers in and
 * out; returns when `vis_out` is written.  `freq` in Hz. */
int hv_vis_gpu(hv_context* ctx, int precision, int method,
               const void* antpos, int nant, double freq,
               const void* eq2tops, int ntimes,
               const void* crd_eq, const void* I_sky, int nsrc,
               const void* bm_cube, int beam_px, void* vis_out);

/* Several frequencies in one call (the reference loops vis_gpu once per
 * frequency, each call with that frequency's beam cube, vis.py:144).
 * freqs: host array (nfreq,) Hz.  Host buffers in and out. */
int hv_vis_multifreq(hv_context* ctx, int precision, int method,
                     const void* antpos, int nant,
                     const double* freqs, int nfreq,
                     const void* eq2tops, int ntimes,
                     const void* crd_eq, const void* I_sky, int nsrc,
                     const void* bm_cubes, int beam_px, void* vis_out);

/* As hv_vis_multifreq with every array already in device memory (freqs
 * stays a host array).  Work is ordered on `stream` (a cudaStream_t; NULL =
 * the context's stream) and the call returns without synchronising; call
 * hv_sync() before reading `d_vis_out` on another stream or the host (the
 * context's stream is made to wait for the call's work on `stream`, unless
 * `stream` is being captured into a graph; then synchronise `stream`
 * itself). */
int hv_vis_multifreq_device(hv_context* ctx, int precision, int method,
                            const void* d_antpos, int nant,
                            const double* freqs, int nfreq,
                            const void* d_eq2tops, int ntimes,
                            const void* d_crd_eq, const void* d_I_sky, int nsrc,
                            const void* d_bm_cubes, int beam_px,
                            void* d_vis_out, void* stream);

/* Wait for the context's work and report any deferred device-side error
 * (e.g. HV_ERR_TIMEOUT from a bounded wait). */
int hv_sync(hv_context* ctx);

/* Device timing of the visibility-product kernels (the fused tensor-core
 * kernel, or the SIMT Hermitian product of the plain form): with profiling
 * on, every launch of them is bracketed by CUDA events on the stream it runs
 * on.  hv_profile_read() synchronises, returns the summed milliseconds and
 * launch count since the previous read, and clears them. */
int hv_set_profiling(hv_context* ctx, int enable);
int hv_profile_read(hv_context* ctx, double* ms, uint64_t* launches);

/* Limit of each device-side wait of the fused kernel in this context
 * (wait_ns = 0: 10 s), and fault injection for tests of failure detection:
 * with stall set, the next fused launches never issue their first source
 * copy, so their consumers' bounded waits run out and the call returns
 * HV_ERR_TIMEOUT with the context still usable.  No counterpart in the
 * reference (it has no device-side waits, hera_gpu/vis.py:144-250). */
int hv_set_wait_limit(hv_context* ctx, uint64_t wait_ns, int stall);

/* Launch shape of the fused kernel for this context's later calls (the
 * batched form takes the same knobs from its autotuner).  No counterpart in
 * the reference, whose launch geometry is a fixed formula (vis.py:176-180).
 * value 0 restores the default of `param`:
 *   HV_TUNE_STAGES      cap on the operand stages held in shared memory,
 *                       2..8 (default: as many as fit; never below the
 *                       number of generator teams).  Fewer stages leave more
 *                       of the SM's on-chip memory to the L1 cache that
 *                       serves the beam gathers. */
enum {
  HV_TUNE_STAGES = 2
};
int hv_set_tuning(hv_context* ctx, int param, int value);

/* ---- batched form -------------------------------------------------------
 * Many independent simulations (precision 1, fused tensor-core form) planned
 * and run together: the reference's per-call vis_gpu (vis.py:144-262) applied
 * to a list of (layout, sky, beams, frequencies) without a host loop.  Every
 * array of an hv_sim is in device memory except `freqs` (host, copied at
 * plan time); the output is (nfreq, ntimes, nant, nant) complex64. */
typedef struct {
  const float* antpos;    /* (nant, 3)            */
  const float* eq2tops;   /* (ntimes, 3, 3)       */
  const float* crd_eq;    /* (3, nsrc)            */
  const float* I_sky;     /* (nsrc,)              */
  const float* bm_cubes;  /* (nfreq, nant, P, P)  */
  const double* freqs;    /* (nfreq,) host, Hz    */
  void* vis_out;          /* (nfreq, ntimes, nant, nant) complex64 */
  int nant, ntimes, nsrc, nfreq, beam_px;
} hv_sim;

typedef struct hv_batch hv_batch;

enum {
  HV_BATCH_GRAPH = 1,     /* capture the batch into a CUDA graph at creation  */
  HV_BATCH_AUTOTUNE = 2   /* time split-K depths per cluster class, keep best */
};

/* Plan a batch on the context's device: one workspace for all simulations,
 * one persistent fused launch per cluster class.  The hv_sim arrays must
 * stay at the same addresses for the life of the batch (a graph replays
 * them).  Runs the batch once when autotuning. */
int hv_batch_create(hv_context* ctx, const hv_sim* sims, int nsims, unsigned flags,
                    hv_batch** batch);
/* Enqueue one run of the batch on `stream` (NULL = the context's stream). */
int hv_batch_launch(hv_batch* batch, void* stream);
/* Wait for the device and report a device-side error of the batch. */
int hv_batch_sync(hv_batch* batch);
/* Kernel launches in one run of the batch. */
uint64_t hv_batch_launches(const hv_batch* batch);
int hv_batch_destroy(hv_batch* batch);
/* Plan, run once, wait, free. */
int hv_vis_batch(hv_context* ctx, const hv_sim* sims, int nsims, void* stream);

/* No counterpart in the reference: an entry point for callers that cannot
 * allocate device memory when they ask for visibilities (a real-time
 * pipeline whose device memory is fixed before it starts, or a framework
 * that owns the allocator).  Single frequency, precision 1, the plain form
 * of the path (same kernels as hv_vis_multifreq_device with
 * HV_METHOD_PLAIN); all inputs and the output (complex64 (ntimes, nant,
 * nant)) are device pointers supplied by the caller, and the call allocates
 * nothing: its working memory is one 64 MiB array per device, held from
 * library load to process exit.  Requests needing more return HV_ERR_ARG
 * with the byte count in `errbuf` (NUL-terminated, up to `errlen` bytes).
 * The first call on a device looks the array up (make it before any stream
 * capture); calls that overlap on the GPU share the array and race, so
 * order them.  Asynchronous on `stream` (NULL = the legacy default stream);
 * no context needed. */
int hv_vis_gpu_noalloc(const void* d_antpos, int nant, double freq,
                       const void* d_eq2tops, int ntimes,
                       const void* d_crd_eq, const void* d_I_sky, int nsrc,
                       const void* d_bm_cube, int beam_px, void* d_vis_out,
                       void* stream, char* errbuf, size_t errlen);

/* ---- 2-D median filter ---------------------------------------------------
 * hera_gpu's MedianFilter (hera_gpu/median_filter.py:8-365): for each of
 * nimg float32 images of rows x cols (C order, one after the other), each
 * output pixel is the element of rank floor(k0 * k1 / 2) (0-based, ascending)
 * of the k0 x k1 window (rows x columns) centred on it, with the image padded
 * by zeros (median_filter.py:318; the window of pixel (r, c) starts at
 * (r - k0/2, c - k1/2)).  For odd windows this is scipy.signal.medfilt2d.
 * Windows whose block tile exceeds 200 KB of shared memory return
 * HV_ERR_ARG.  The _device form takes device buffers and returns without
 * synchronising (stream NULL = the context's stream). */
int hv_median_filter(hv_context* ctx, const float* in, float* out, int nimg, int rows, int cols,
                     int k0, int k1);
int hv_median_filter_device(hv_context* ctx, const float* d_in, float* d_out, int nimg,
                            int rows, int cols, int k0, int k1, void* stream);

/* ---- Omnical redundant calibration --------------------------------------
 * hera_gpu's omnical (hera_gpu/redcal.py:358-743): for each of ndata
 * independent problems p, iterate the Omnical solution of
 *   data[p][b] = gains[p][i_b] * conj(gains[p][j_b]) * ubls[p][k_b]
 * with (i_b, j_b, k_b) = ggu[3 b .. 3 b + 2] (a HOST array of nbls uint32
 * triples, redcal.py:392-393,423), as the reference's kernels do
 * (redcal.py:70-354): weights every check_every iterations, a step of
 * fraction `gain` toward the new estimate each iteration, and a
 * convergence / chi^2 check every check_every iterations from check_after on
 * and at maxiter (redcal.py:587-702).  precision 1: complex64 gains, ubls
 * and data, float32 wgts, chisq and conv; precision 2: complex128 / float64.
 * gains (ndata x nants) and ubls (ndata x nubls) are overwritten with the
 * solutions; chisq, iters (the last accepted iteration, 0 if none) and conv
 * (the last relative change) get one value per problem (redcal.py:742).
 * check_every must be > 1 (redcal.py:402), nants <= 65535; a triple out of
 * range returns HV_ERR_ARG.  The _device form takes device buffers (ggu
 * still on the host) and returns without synchronising (stream NULL = the
 * context's stream). */
int hv_omnical(hv_context* ctx, int precision, const uint32_t* ggu, int nbls, void* gains,
               int nants, void* ubls, int nubls, const void* data, const void* wgts, int ndata,
               double conv_crit, int maxiter, int check_every, int check_after, double gain,
               void* chisq, uint32_t* iters, void* conv);
int hv_omnical_device(hv_context* ctx, int precision, const uint32_t* ggu, int nbls,
                      void* d_gains, int nants, void* d_ubls, int nubls, const void* d_data,
                      const void* d_wgts, int ndata, double conv_crit, int maxiter,
                      int check_every, int check_after, double gain, void* d_chisq,
                      uint32_t* d_iters, void* d_conv, void* stream);

/* Device memory and copies ordered on the context's stream (stream-ordered
 * allocation, so freeing does not stall other streams); used by host code
 * that keeps inputs resident or serves requests.  kind: 1 host->device,
 * 2 device->host, 3 device->device.  Replace the PyCUDA gpuarray.to_gpu /
 * gpuarray.empty buffers, .set() uploads and driver.Stream of
 * hera_gpu/vis.py:198-209,214. */
int hv_device_alloc(hv_context* ctx, size_t bytes, void** ptr);
int hv_device_free(hv_context* ctx, void* ptr);
int hv_memcpy_async(hv_context* ctx, void* dst, const void* src, size_t bytes, int kind);
/* 0 when every operation queued on the context's stream has finished, 1 while
 * work is pending; a negative hv_status on error. */
int hv_stream_query(hv_context* ctx);

/* Page-locked host memory for fast host<->device copies (cudaHostAlloc);
 * replaces the host download buffers of hera_gpu/vis.py:207-208. */
int hv_host_alloc(hv_context* ctx, size_t bytes, void** ptr);
int hv_host_free(hv_context* ctx, void* ptr);

#ifdef __cplusplus
}
#endif
#endif /* HERAVIS_H */
