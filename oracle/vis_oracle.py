"""CPU oracle for the visibility simulator -- TEST INFRASTRUCTURE ONLY.

This module is the checker, never the product.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import it.  The product path (``hera_gpu_gb300``) never calls it and fails
loudly when its CUDA library is missing.

What it restates
----------------
The reference's own CPU implementation of the measurement equation,
``vis_cpu`` in ``hera_gpu/tests/test_vis_gpu.py:278-357``:

* cast inputs to the working real dtype (test_vis_gpu.py:314-324);
* per time: ``crd_top = eq2top @ crd_eq`` (test_vis_gpu.py:331);
* per antenna: bilinear interpolation of ``bm_cube[i]`` on the grid
  ``linspace(-1, 1, P)`` at ``(ty, tx)`` (test_vis_gpu.py:326-335).  The
  reference calls ``scipy.interpolate.RectBivariateSpline(kx=1, ky=1)``;
  that spline is piecewise bilinear and clamps outside the grid, which is
  what :func:`bilinear_beam` computes in closed form (pinned against scipy in
  ``tests/test_oracle.py``);
* horizon mask ``A = 0`` where ``tz <= 0`` (test_vis_gpu.py:336);
* ``tau = antpos @ crd_top / c``, ``v = A * sqrt(I) * exp(+i 2 pi nu tau)``
  (test_vis_gpu.py:339-344), c = 299 792 458 m/s (astropy's value);
* ``vis[t, a, b] = sum_s v[a, s] * conj(v[b, s])``: the reference forms the
  upper triangle with ``conj(v_i) . v_j``, conjugates, and mirrors the lower
  triangle (test_vis_gpu.py:347-355); the result is the full Hermitian matrix
  with a real diagonal.

Parity is pinned: ``tests/golden/make_golden.py`` ran the reference's
``vis_cpu`` itself (imported from the reference sources with its GPU-only
imports stubbed) and stored inputs and outputs under ``tests/golden/``;
``tests/test_oracle.py`` checks this module against those fixtures and
against the reference's known-answer tests (test_vis_gpu.py:203-244).
"""
from __future__ import annotations

import numpy as np

SPEED_OF_LIGHT = 299792458.0  # m/s, astropy.constants.c (vis.py:4,8)


def bilinear_beam(beam: np.ndarray, x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """Bilinear interpolation of one beam map ``beam[y_idx, x_idx]`` on the
    grid ``linspace(-1, 1, P)`` for both axes, clamped at the edges.

    Restates ``RectBivariateSpline(bm_pix_y, bm_pix_x, bm_cube[i], kx=1,
    ky=1)(ty, tx, grid=False)`` (test_vis_gpu.py:334-335) and the texture
    lookup of ``InterpolateBeam`` (vis.py:63-84): fractional pixel
    ``b = (P-1)(0.5 x + 0.5)``, corner ``floor(b)``, weight ``b - floor(b)``;
    outside the grid both return the edge value.
    """
    P = beam.shape[-1]
    dt = beam.dtype
    bx = (P - 1) * (0.5 * x.astype(dt) + 0.5)
    by = (P - 1) * (0.5 * y.astype(dt) + 0.5)
    px = np.floor(bx)
    py = np.floor(by)
    fx = bx - px
    fy = by - py
    px = px.astype(np.int64)
    py = py.astype(np.int64)
    x0 = np.clip(px, 0, P - 1)
    x1 = np.clip(px + 1, 0, P - 1)
    y0 = np.clip(py, 0, P - 1)
    y1 = np.clip(py + 1, 0, P - 1)
    b00 = beam[..., y0, x0]
    b01 = beam[..., y0, x1]
    b10 = beam[..., y1, x0]
    b11 = beam[..., y1, x1]
    top = b00 + fx * (b01 - b00)
    bot = b10 + fx * (b11 - b10)
    return top + fy * (bot - top)


def phasors(antpos, freq, eq2top, crd_eq, I_sky, bm_cube, dtype=np.float64):
    """Per-antenna, per-source complex voltages ``v[a, s]`` for one time.

    Restates test_vis_gpu.py:331-344 (the body of the time loop up to the
    visibility product).  Returns complex (nant, nsrc).
    """
    rt = np.dtype(dtype)
    ct = np.result_type(rt, np.complex64)
    antpos = np.asarray(antpos).astype(rt)
    eq2top = np.asarray(eq2top).astype(rt)
    crd_eq = np.asarray(crd_eq).astype(rt)
    Isqrt = np.sqrt(np.asarray(I_sky)).astype(rt)
    bm = np.asarray(bm_cube).astype(rt)
    tx, ty, tz = crd_top = eq2top @ crd_eq
    A = np.empty((bm.shape[0], crd_eq.shape[1]), dtype=rt)
    for i in range(bm.shape[0]):
        A[i] = bilinear_beam(bm[i], tx, ty)
    A = np.where(tz > 0, A, 0).astype(rt)
    tau = (antpos @ crd_top) * rt.type(1.0 / SPEED_OF_LIGHT)
    ang = rt.type(2 * np.pi * freq)
    v = np.exp((1j * ang) * tau).astype(ct)
    v *= A * Isqrt
    return v


def hermitian_product(v: np.ndarray) -> np.ndarray:
    """``V[a, b] = sum_s v[a, s] conj(v[b, s])`` with the reference's
    orientation (test_vis_gpu.py:347-355): upper triangle computed, lower
    triangle the conjugate mirror, diagonal real."""
    V = v @ v.conj().T
    n = V.shape[0]
    iu = np.triu_indices(n, 1)
    V[iu[1], iu[0]] = V[iu].conj()
    V[np.diag_indices(n)] = V.diagonal().real
    return V


def vis_oracle(antpos, freq, eq2tops, crd_eq, I_sky, bm_cube, dtype=np.float64):
    """Full oracle: ``vis[t, a, b]`` for every time in ``eq2tops``.

    ``dtype`` is the working real dtype (float64 is the FP64 oracle used for
    every parity check; float32 mimics ``vis_cpu(precision=1)``).
    """
    rt = np.dtype(dtype)
    ct = np.result_type(rt, np.complex64)
    nant = np.asarray(antpos).shape[0]
    ntimes = np.asarray(eq2tops).shape[0]
    out = np.empty((ntimes, nant, nant), dtype=ct)
    for t in range(ntimes):
        v = phasors(antpos, freq, eq2tops[t], crd_eq, I_sky, bm_cube, rt)
        out[t] = hermitian_product(v)
    return out


def vis_oracle_partial(antpos, freq, eq2top, crd_eq, I_sky, bm_cube, s0, s1,
                       dtype=np.float64):
    """One time, sources ``[s0, s1)`` only: the un-mirrored ``v @ v^H`` sum
    over that slice (used to time bounded samples and to split work across
    host processes; summing slices gives :func:`vis_oracle` up to rounding)."""
    v = phasors(antpos, freq, eq2top, np.asarray(crd_eq)[:, s0:s1],
                np.asarray(I_sky)[s0:s1], bm_cube, dtype)
    return v @ v.conj().T


def rel_frobenius(a: np.ndarray, ref: np.ndarray, axes=(-2, -1)) -> np.ndarray:
    """Relative Frobenius error ``||a - ref||_F / ||ref||_F`` over the last two
    axes (one value per (time) or (time, frequency) slice)."""
    a = np.asarray(a, dtype=np.complex128)
    ref = np.asarray(ref, dtype=np.complex128)
    num = np.sqrt(np.sum(np.abs(a - ref) ** 2, axis=axes))
    den = np.sqrt(np.sum(np.abs(ref) ** 2, axis=axes))
    return num / np.where(den == 0, 1.0, den)
