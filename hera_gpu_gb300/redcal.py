"""Drop-in for hera_gpu's Omnical solver (``hera_gpu.redcal.omnical``).

The reference (hera_gpu/redcal.py:358-743) solves many independent Omnical
problems -- one per "pixel" (frequency x time sample) -- 64 at a time, with
a dozen kernel launches per iteration and a host round trip at every
convergence check.  Here every problem of the call goes through one launch of
libheravis.so's omnical kernel (``hv_omnical``): one CTA per problem, all
iterations inside the kernel, deterministic sums.

The ``OmnicalSolverGPU`` / ``RedundantCalibratorGPU`` wrappers of the
reference (redcal.py:746-883) subclass ``hera_cal`` classes; ``hera_cal`` is
not a dependency of this package, so they are not provided here -- a caller
of those classes passes their arrays to ``omnical`` below, exactly as
redcal.py:799-820 does.
"""
from __future__ import annotations

import numpy as np

from . import _native

NTHREADS = 1024


def omnical(ggu_indices, gains, ubls, data, wgts, conv_crit=1e-10, maxiter=50, check_every=4,
            check_after=1, gain=0.3, nthreads=NTHREADS, precision=1, verbose=False,
            context=None):
    """Omnical iterations for ``ndata`` independent problems.

    Args (as hera_gpu.redcal.omnical, redcal.py:358-389):
        ggu_indices: (nbls, 3) indices (i, j, k): data = gains[i] gains[j]* ubls[k]
        gains: (ndata, nants) starting gains
        ubls: (ndata, nubls) starting unique-baseline visibilities
        data: (ndata, nbls) data; wgts: (ndata, nbls) weights
        conv_crit, maxiter, check_every, check_after, gain: as the reference
        nthreads: accepted and not needed (the library picks its launch)
        precision: 1 = float32 / complex64, 2 = float64 / complex128

    Returns {'gains', 'ubls', 'chisq', 'iters', 'conv'} (new arrays; the
    inputs are not modified, as the reference's astype copies).
    """
    nbls = ggu_indices.shape[0]
    assert ggu_indices.shape == (nbls, 3)
    ndata = data.shape[0]
    assert data.shape == (ndata, nbls)
    assert wgts.shape == (ndata, nbls)
    nants = gains.shape[1]
    assert gains.shape == (ndata, nants)
    nubls = ubls.shape[1]
    assert ubls.shape == (ndata, nubls)
    assert precision in (1, 2)
    assert check_every > 1
    if verbose:
        print("PRECISION:", precision)
        print("NDATA:", ndata)
        print("NANTS:", nants)
        print("NUBLS:", nubls)
        print("NBLS:", nbls)
    rt, ct = (np.float32, np.complex64) if precision == 1 else (np.float64, np.complex128)
    ggu = np.ascontiguousarray(ggu_indices, dtype=np.uint32)
    data = np.ascontiguousarray(data, dtype=ct)
    wgts = np.ascontiguousarray(wgts, dtype=rt)
    gains = np.array(gains, dtype=ct, order="C", copy=True)
    ubls = np.array(ubls, dtype=ct, order="C", copy=True)
    chisq = np.empty((ndata,), dtype=rt)
    conv = np.empty((ndata,), dtype=rt)
    iters = np.empty((ndata,), dtype=np.uint32)
    ctx = context or _native.default_context()
    ctx.omnical(precision, ggu, gains, ubls, data, wgts, conv_crit, maxiter, check_every,
                check_after, gain, chisq, iters, conv)
    return {"gains": gains, "ubls": ubls, "chisq": chisq, "iters": iters, "conv": conv}
