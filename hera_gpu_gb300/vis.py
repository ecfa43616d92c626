"""Drop-in replacement for ``hera_gpu.vis.vis_gpu`` (reference
``hera_gpu/vis.py:144-262``) on GB300.

``vis_gpu(antpos, freq, eq2tops, crd_eq, I_sky, bm_cube, ...)`` keeps the
reference's arguments, shape checks (AssertionError, vis.py:147,161-169),
dtype rules (vis.py:147-157, 171-175) and output: a new host array
``(ntimes, nant, nant)`` holding the full Hermitian matrix
``V[a, b] = sum_s v[a, s] conj(v[b, s])``.  It also accepts the
``real_dtype`` / ``complex_dtype`` spelling of ``vis_cpu``-style callers.

Differences that are fixes, not choices:
* every source is used (the reference drops ``npix mod chunk`` sources,
  vis.py:176-177);
* the phase ``2 pi nu tau`` is reduced to cycles with FP64-class accuracy in
  every precision, so long baselines keep their phase.

``nthreads`` and ``max_memory`` are accepted for signature compatibility; the
launch geometry and workspace are chosen by the library.
"""
from __future__ import annotations

import numpy as np

from . import _native

ONE_OVER_C = 1.0 / 299792458.0   # s/m (vis.py:8); the library's delays use the same c
NTHREADS = 1024          # reference module constants (vis.py:140-142), accepted only
MAX_MEMORY = 2 ** 29
MIN_CHUNK = 8


def _as_dtype(x, name):
    """np.dtype(x), or an AssertionError naming the argument: a reference
    caller passing ``nthreads`` positionally lands an integer here."""
    try:
        return np.dtype(x)
    except TypeError:
        raise AssertionError(f"{name} must be a dtype (got {x!r}); nthreads, max_memory, "
                             "precision and verbose are keyword arguments here") from None


def _resolve_precision(precision, real_dtype, complex_dtype):
    if real_dtype is not None:
        real_dtype = _as_dtype(real_dtype, "real_dtype")
    if complex_dtype is not None:
        complex_dtype = _as_dtype(complex_dtype, "complex_dtype")
    if precision is None:
        if real_dtype is not None:
            precision = 2 if np.dtype(real_dtype) == np.float64 else 1
        elif complex_dtype is not None:
            precision = 2 if np.dtype(complex_dtype) == np.complex128 else 1
        else:
            precision = 1
    assert precision in (1, 2)
    if real_dtype is not None:
        assert np.dtype(real_dtype) == (np.float32 if precision == 1 else np.float64)
    if complex_dtype is not None:
        assert np.dtype(complex_dtype) == (np.complex64 if precision == 1 else np.complex128)
    if precision == 1:
        return 1, np.float32, np.complex64
    return 2, np.float64, np.complex128


def _check_shapes(antpos, eq2tops, crd_eq, I_sky, bm_cubes, multifreq):
    nant = antpos.shape[0]
    assert antpos.shape == (nant, 3)
    npix = crd_eq.shape[1]
    assert crd_eq.shape == (3, npix)
    assert I_sky.shape == (npix,)
    beam_px = bm_cubes.shape[-2]
    if multifreq:
        assert bm_cubes.ndim == 4 and bm_cubes.shape[1:] == (nant, beam_px, beam_px)
    else:
        assert bm_cubes.shape == (nant, beam_px, beam_px)
    ntimes = eq2tops.shape[0]
    assert eq2tops.shape == (ntimes, 3, 3)
    return nant, npix, ntimes, beam_px


def vis_gpu(antpos, freq, eq2tops, crd_eq, I_sky, bm_cube, real_dtype=None,
            complex_dtype=None, nthreads=NTHREADS, max_memory=MAX_MEMORY, precision=None,
            verbose=False, method="auto", context=None):
    """Visibilities of a point-source sky for one frequency.

    Args (as the reference):
        antpos (nant, 3): antenna positions [m].
        freq (float): frequency [Hz] (phase = 2 pi freq tau, tau in s).
        eq2tops (ntimes, 3, 3): equatorial -> topocentric rotations.
        crd_eq (3, nsrc): equatorial unit vectors of the sources.
        I_sky (nsrc,): source intensities.
        bm_cube (nant, P, P): beam power on the grid linspace(-1, 1, P),
            axes [ant, y(m), x(l)].
        real_dtype / complex_dtype or precision: float32/complex64 (1) or
            float64/complex128 (2).
        method: "auto" (tensor-core form for precision 1), "plain" (the
            reference's method, FP32/FP64 SIMT product), or "tc".
    Returns:
        ndarray (ntimes, nant, nant) of complex_dtype.
    """
    antpos = np.asarray(antpos)
    eq2tops = np.asarray(eq2tops)
    crd_eq = np.asarray(crd_eq)
    I_sky = np.asarray(I_sky)
    bm_cube = np.asarray(bm_cube)
    prec, rt, ct = _resolve_precision(precision, real_dtype, complex_dtype)
    nant, npix, ntimes, beam_px = _check_shapes(antpos, eq2tops, crd_eq, I_sky, bm_cube, False)
    out = np.empty((1, ntimes, nant, nant), dtype=ct)
    ctx = context or _native.default_context()
    ctx.vis_multifreq(prec, method,
                      np.ascontiguousarray(antpos, dtype=rt), np.array([float(freq)]),
                      np.ascontiguousarray(eq2tops, dtype=rt), np.ascontiguousarray(crd_eq, dtype=rt),
                      np.ascontiguousarray(I_sky, dtype=rt),
                      np.ascontiguousarray(bm_cube, dtype=rt)[None], out)
    return out[0]


def vis_gpu_multifreq(antpos, freqs, eq2tops, crd_eq, I_sky, bm_cubes, real_dtype=None,
                      complex_dtype=None, precision=None, method="auto", context=None, out=None):
    """Several frequencies in one call: ``bm_cubes`` (nfreq, nant, P, P) ->
    ``(nfreq, ntimes, nant, nant)``.  Equal to stacking ``vis_gpu`` per
    frequency (how the reference is driven for more than one channel), with
    the source rotation and horizon cut shared across frequencies.  ``out``
    may supply the (nfreq, ntimes, nant, nant) result array (e.g. in
    page-locked memory)."""
    antpos = np.asarray(antpos)
    eq2tops = np.asarray(eq2tops)
    crd_eq = np.asarray(crd_eq)
    I_sky = np.asarray(I_sky)
    bm_cubes = np.asarray(bm_cubes)
    freqs = np.atleast_1d(np.asarray(freqs, dtype=np.float64))
    prec, rt, ct = _resolve_precision(precision, real_dtype, complex_dtype)
    nant, npix, ntimes, beam_px = _check_shapes(antpos, eq2tops, crd_eq, I_sky, bm_cubes, True)
    assert bm_cubes.shape[0] == len(freqs)
    if out is None:
        out = np.empty((len(freqs), ntimes, nant, nant), dtype=ct)
    assert out.shape == (len(freqs), ntimes, nant, nant) and out.dtype == ct
    assert out.flags.c_contiguous
    ctx = context or _native.default_context()
    ctx.vis_multifreq(prec, method,
                      np.ascontiguousarray(antpos, dtype=rt), freqs,
                      np.ascontiguousarray(eq2tops, dtype=rt), np.ascontiguousarray(crd_eq, dtype=rt),
                      np.ascontiguousarray(I_sky, dtype=rt), np.ascontiguousarray(bm_cubes, dtype=rt),
                      out)
    return out
