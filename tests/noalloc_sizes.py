"""Working memory of hv_vis_gpu_noalloc for a request, restated from
hera_gpu_gb300/csrc/hv_noalloc.cu so that tests can pick requests at its
limit: every region rounded up to 256 bytes, in the order the call lays
them out (frequency, transposed beam, phase coefficients, counts, prep
block counts, source records, phasors, split-K partial sums)."""

SCRATCH_BYTES = 64 << 20   # kNoAllocScratchBytes
PLAIN_CHUNK = 4096         # kPlainChunk (hv_kernels.h)
ANT_PAD = 128              # kAntPad (hv_internal.cuh)
PREP_BLOCK = 1024          # kPrepBlock (hv_internal.cuh)


def up256(x):
    return (x + 255) & ~255


def need_bytes(nant, nsrc, ntimes, beam_px):
    np_ = -(-nant // ANT_PAD) * ANT_PAD
    s1 = max(nsrc, 1)
    chunks = -(-s1 // PLAIN_CHUNK)
    prep_blocks = -(-nsrc // PREP_BLOCK) if nsrc > 0 else 1
    return (up256(8) + up256(4 * beam_px * beam_px * np_) + up256(32 * ntimes * np_)
            + up256(4 * ntimes) + up256(4 * prep_blocks) + up256(32 * s1)
            + up256(8 * s1 * np_) + up256(4 * chunks * 2 * np_ * np_))


def largest_nsrc(nant, ntimes, beam_px):
    """The most sources a request of this shape may have (need is monotone
    in nsrc)."""
    lo, hi = 0, 1
    while need_bytes(nant, hi, ntimes, beam_px) <= SCRATCH_BYTES:
        lo, hi = hi, 2 * hi
    while hi - lo > 1:
        mid = (lo + hi) // 2
        if need_bytes(nant, mid, ntimes, beam_px) <= SCRATCH_BYTES:
            lo = mid
        else:
            hi = mid
    return lo
