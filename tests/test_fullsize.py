"""Parity at the benchmark's sizes.

* Array scale (350 antennas, 100,000 sources, 63 x 63 Airy beams): every
  method against the FP64 oracle on the same inputs, at the tolerances of
  test_vis_parity.py.
* The precision form's full size (350 antennas, 1,048,576 sources, 64
  channels over 100-200 MHz with per-channel beams), where the FP64 oracle of
  the whole product is out of reach, through properties that do not depend
  on the size:
    - the output is Hermitian bit for bit, with a real, positive diagonal;
    - the autocorrelations V[a, a] = sum over sources above the horizon of
      A_a(l, m)^2 I carry no phase, so the oracle computes them at full size
      (beam interpolation only);
    - the product is linear in the sources: the visibilities of all sources
      equal the sum of those of two halves;
  and through whole slices against the FP64 oracle, cross-correlations
  included: the lowest channel (100 MHz) at the first LST and the highest
  (200 MHz, twice the phase range) at the second, every one of the 1,048,576
  sources (the oracle sums them in blocks to bound its memory).
"""
import numpy as np
import pytest

from hera_gpu_gb300 import synth, vis_gpu, vis_gpu_multifreq
from oracle import bilinear_beam, rel_frobenius, vis_oracle, vis_oracle_partial

pytestmark = pytest.mark.gpu


def as_seen(x, precision=1):
    return np.asarray(x).astype(np.float32 if precision == 1 else np.float64).astype(np.float64)


@pytest.fixture(scope="module")
def full():
    cfg = synth.config_array(seed=0, nant=350, nsrc=1_048_576, ntimes=2, nfreq=64, fmin=100e6,
                             fmax=200e6, P=63)
    bm = synth.beams_for(cfg, dtype=np.float32)
    args = (cfg["antpos"].astype(np.float32), cfg["freqs"], cfg["eq2tops"].astype(np.float32),
            cfg["crd_eq"].astype(np.float32), cfg["I_sky"].astype(np.float32), bm)
    V = vis_gpu_multifreq(*args, precision=1, method="tc")
    V16 = vis_gpu_multifreq(*args, precision=1, method="tc_fp16")
    return args, V, V16


def test_fullsize_hermitian(full):
    _, V, _ = full
    assert V.shape == (64, 2, 350, 350) and V.dtype == np.complex64
    np.testing.assert_array_equal(V, np.conj(np.swapaxes(V, -1, -2)))
    d = np.diagonal(V, axis1=-2, axis2=-1)
    assert np.all(d.imag == 0) and np.all(d.real > 0)


@pytest.mark.parametrize("t,f", [(0, 0), (1, 63)])
def test_fullsize_autocorrelations(full, t, f):
    (antpos, freqs, e2t, crd, I, bm), V, V16 = full
    top = as_seen(e2t[t]) @ as_seen(crd)
    up = top[2] > 0
    tx, ty = top[0, up], top[1, up]
    Iu = as_seen(I)[up]
    beams = as_seen(bm[f])
    ref = np.array([np.dot(bilinear_beam(beams[a], tx, ty) ** 2, Iu) for a in range(350)])
    for out in (V, V16):
        got = np.diagonal(out[f, t]).real.astype(np.float64)
        err = np.abs(got - ref) / ref
        assert err.max() <= 1e-4, err.max()


def oracle_slice(args, t, f, block=131072):
    """FP64 oracle of slice (t, f) of the full-size call over all sources, in
    the library's orientation (upper triangle computed, lower its conjugate)."""
    antpos, freqs, e2t, crd, I, bm = args
    a64 = lambda x: np.asarray(x, dtype=np.float64)
    V = 0
    for s0 in range(0, crd.shape[1], block):
        V = V + vis_oracle_partial(a64(antpos), float(freqs[f]), a64(e2t[t]), a64(crd[:, s0:s0 + block]),
                                   a64(I[s0:s0 + block]), a64(bm[f]), 0, min(block, crd.shape[1] - s0))
    return np.triu(V) + np.triu(V, 1).conj().T


@pytest.mark.parametrize("t,f", [(0, 0), (1, 63)])
def test_fullsize_slice_against_oracle(full, t, f):
    args, V, V16 = full
    ref = oracle_slice(args, t, f)
    for name, out in (("tc", V), ("tc_fp16", V16)):
        err = rel_frobenius(out[f, t], ref)
        assert err <= 1e-4, (name, err)


def test_fullsize_linear_in_the_sources(full):
    (antpos, freqs, e2t, crd, I, bm), V, _ = full
    chans = np.arange(0, 64, 8)
    h = crd.shape[1] // 2
    part = lambda s: vis_gpu_multifreq(antpos, freqs[chans], e2t[:1], crd[:, s],
                                       np.ascontiguousarray(I[s]), bm[chans], precision=1,
                                       method="tc")
    both = part(slice(0, h)).astype(np.complex128) + part(slice(h, None))
    err = rel_frobenius(both, V[chans, :1]).max()
    assert err <= 1e-4, err


_ARRAY = {}


def array_scale(precision):
    """Config-2 inputs (two of its 60 LSTs: the first and the last) in the
    precision's dtype, and the FP64 oracle on exactly those inputs."""
    if precision not in _ARRAY:
        cfg = synth.config_array(seed=2, nant=350, nsrc=100_000, ntimes=60, nfreq=1,
                                 fmin=150e6, fmax=150e6, P=63)
        bm = synth.beams_for(cfg, dtype=np.float64)[0]
        rt = np.float32 if precision == 1 else np.float64
        args = (cfg["antpos"].astype(rt), 150e6, cfg["eq2tops"][[0, 59]].astype(rt),
                cfg["crd_eq"].astype(rt), cfg["I_sky"].astype(rt), bm.astype(rt))
        ref = vis_oracle(*(as_seen(a, precision) if isinstance(a, np.ndarray) else a
                           for a in args))
        _ARRAY[precision] = (args, ref)
    return _ARRAY[precision]


@pytest.mark.parametrize("method,precision,tol", [("plain", 1, 1e-5), ("tc", 1, 1e-4),
                                                  ("tc_fp16", 1, 1e-4), ("plain", 2, 1e-11)])
def test_array_scale_against_oracle(method, precision, tol):
    args, ref = array_scale(precision)
    V = vis_gpu(*args, precision=precision, method=method)
    err = rel_frobenius(V, ref).max()
    assert err <= tol, err
