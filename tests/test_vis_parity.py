"""GPU parity of every method against the oracle and the reference's fixtures.

Tolerances (relative Frobenius error per time slice, vs the FP64 oracle run
on the same inputs as the GPU saw):
    plain,   precision 1 (FP32 SIMT product)                    <= 1e-5
    tc,      precision 1 (split-BF16 tensor cores)              <= 1e-4
    tc_fp16, precision 1 (FP16 + E4M3 split, tensor cores)      <= 1e-4
    plain,   precision 2 (FP64)                                 <= 1e-11
The FP64 bound is set by FP64 rounding of phases of ~1e3 cycles (the
km-baseline fixture), where the oracle itself carries errors of 1e-12.
"""
import os

import numpy as np
import pytest

from hera_gpu_gb300 import synth, vis_gpu, vis_gpu_multifreq
from oracle import rel_frobenius, vis_oracle
from vis_gpu_cases import VIS_GPU_CASES, load_vis_gpu_case

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL = {("plain", 1): 1e-5, ("tc", 1): 1e-4, ("tc_fp16", 1): 1e-4, ("plain", 2): 1e-11,
       ("auto", 1): 1e-4, ("auto", 2): 1e-11}
METHODS = [("plain", 1), ("plain", 2), ("tc", 1), ("tc_fp16", 1)]


def as_seen(x, precision):
    """The inputs exactly as the GPU path sees them (cast to its real dtype)."""
    return np.asarray(x).astype(np.float32 if precision == 1 else np.float64).astype(np.float64)


def oracle_same_inputs(args, precision):
    antpos, freq, e2t, crd, I, bm = args
    return vis_oracle(as_seen(antpos, precision), freq, as_seen(e2t, precision),
                      as_seen(crd, precision), as_seen(I, precision), as_seen(bm, precision))


def load(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    return (d["antpos"], float(d["freq"]), d["eq2tops"], d["crd_eq"], d["I_sky"], d["bm_cube"]), d


@pytest.mark.parametrize("method,precision", METHODS)
@pytest.mark.parametrize("name", ["small_config", "random_inputs", "edge_inputs"])
def test_golden_fixtures(name, method, precision):
    args, d = load(name)
    v = vis_gpu(*args, precision=precision, method=method)
    assert v.dtype == (np.complex64 if precision == 1 else np.complex128)
    assert v.shape == d["vis_p2"].shape
    ref = oracle_same_inputs(args, precision)
    err = rel_frobenius(v, ref)
    assert err.max() <= TOL[(method, precision)], err
    if precision == 2:
        # the reference's own FP64 output (fixture) to FP64 rounding
        assert rel_frobenius(v, d["vis_p2"]).max() < 1e-11
    # Hermitian with a real diagonal, as the reference's mirror step leaves it
    np.testing.assert_array_equal(v, np.conj(np.transpose(v, (0, 2, 1))))
    assert np.all(np.diagonal(v, axis1=1, axis2=2).imag == 0)


@pytest.mark.parametrize("method,precision", METHODS)
@pytest.mark.parametrize("name", VIS_GPU_CASES)
def test_reference_vis_gpu_fixtures(name, method, precision):
    # the reference's own vis_gpu (run on the CPU) on the sources it sums
    used, _, out = load_vis_gpu_case(name)
    v = vis_gpu(*used, precision=precision, method=method)
    assert rel_frobenius(v, oracle_same_inputs(used, precision)).max() <= TOL[(method, precision)]
    if precision == 2:
        assert rel_frobenius(v, out[2]).max() < 1e-11


# --- known answers of test_vis_gpu.py:203-244 -------------------------------
NANT, NTIMES, BM_PIX, NPIX = 16, 10, 31, 12 * 16 ** 2


def kat_inputs():
    antpos = np.ones((NANT, 3))
    eq2tops = np.array([np.identity(3)] * NTIMES)
    crd_eq = np.zeros((3, NPIX))
    crd_eq[2] = 1
    return antpos, eq2tops, crd_eq, np.ones(NPIX), np.ones((NANT, BM_PIX, BM_PIX))


@pytest.mark.parametrize("method,precision", METHODS)
def test_kat_values(method, precision):
    antpos, eq2tops, crd_eq, I_sky, bm = kat_inputs()
    kw = dict(precision=precision, method=method)
    np.testing.assert_equal(vis_gpu(antpos, 1.0, eq2tops, crd_eq, I_sky * 0, bm, **kw), 0)
    np.testing.assert_equal(vis_gpu(antpos, 1.0, eq2tops, crd_eq, I_sky, bm * 0, **kw), 0)
    # co-located antennas, every source at zenith: V = NPIX (decimal 22 in the reference)
    v = vis_gpu(antpos, 1.0, eq2tops, crd_eq, I_sky, bm, **kw)
    np.testing.assert_almost_equal(v, NPIX, 22 if precision == 2 or method == "plain" else 3)
    if method == "tc_fp16":
        # every source at the beam's peak, |X| = 256 exactly: the scaled
        # split is exact, so the sum is too
        np.testing.assert_equal(v, NPIX)
    # two sources, at zenith and at 45 deg: V ~ 2
    crd2 = np.zeros((3, 2))
    crd2[2, 0] = 1
    crd2[1, 1] = np.sqrt(0.5)
    crd2[2, 1] = np.sqrt(0.5)
    v = vis_gpu(antpos, 1.0, eq2tops, crd2, np.ones(2), bm, **kw)
    np.testing.assert_almost_equal(v, 2, 2)
    # one antenna moved: against the oracle (decimal 5 FP32 / 15 FP64 in the reference)
    antpos[0, 0] = 0
    antpos[0, 1] = 0
    v = vis_gpu(antpos, 1.0, eq2tops, crd2, np.ones(2), bm, **kw)
    ref = vis_oracle(antpos, 1.0, eq2tops, crd2, np.ones(2), bm)
    np.testing.assert_almost_equal(v, ref, 15 if precision == 2 else 5)


@pytest.mark.parametrize("method,precision", METHODS)
def test_kat_beam_of_one_centre_pixel(method, precision):
    # test_vis_gpu.py:66-102 through the whole call: a beam of one centre
    # pixel gives A = 1 at zenith (V = the number of sources) and A = 0 at
    # 45 degrees off it (V = 0)
    antpos, eq2tops, crd_eq, I_sky, _ = kat_inputs()
    middle = np.zeros((NANT, BM_PIX, BM_PIX))
    middle[:, BM_PIX // 2, BM_PIX // 2] = 1.0
    kw = dict(precision=precision, method=method)
    v = vis_gpu(antpos, 1.0, eq2tops, crd_eq, I_sky, middle, **kw)
    assert rel_frobenius(v, np.full(v.shape, NPIX, dtype=np.complex128)).max() <= \
        TOL[(method, precision)]
    crd_eq[1] = crd_eq[2] = np.sqrt(0.5)
    np.testing.assert_equal(vis_gpu(antpos, 1.0, eq2tops, crd_eq, I_sky, middle, **kw), 0)


@pytest.mark.parametrize("method,precision", METHODS)
def test_dtypes_and_shapes(method, precision):
    # test_vis_gpu.py:172-202
    v = vis_gpu(np.zeros((NANT, 3)), 0.15, np.zeros((NTIMES, 3, 3)), np.zeros((3, NPIX)),
                np.zeros(NPIX), np.zeros((NANT, BM_PIX, BM_PIX)), precision=precision,
                method=method)
    assert v.shape == (NTIMES, NANT, NANT)
    assert v.dtype == (np.complex64 if precision == 1 else np.complex128)


def test_real_dtype_spelling():
    args, _ = load("small_config")
    a = vis_gpu(*args, real_dtype=np.float64, complex_dtype=np.complex128)
    b = vis_gpu(*args, precision=2)
    np.testing.assert_array_equal(a, b)


# --- edge cases ---------------------------------------------------------------
@pytest.mark.parametrize("method,precision", METHODS)
@pytest.mark.parametrize("nant,nsrc,ntimes,P", [
    (1, 50, 2, 31),      # a single antenna
    (129, 700, 2, 5),    # one past a 128-antenna block
    (37, 1, 3, 2),       # one source, 2-pixel beam
    (20, 300, 1, 1),     # 1-pixel beam
    (8, 0, 2, 31),       # no sources
    (300, 2100, 1, 63),  # several antenna blocks and source chunks
])
def test_edge_sizes(method, precision, nant, nsrc, ntimes, P):
    rng = np.random.default_rng(nant * 1000 + nsrc)
    antpos = rng.normal(0, 100.0, (nant, 3))
    crd = synth.sphere_sources(nsrc, rng)
    I = rng.random(nsrc) * 3
    bm = rng.random((nant, P, P))
    e2t = np.stack([np.linalg.qr(rng.normal(size=(3, 3)))[0] for _ in range(ntimes)])
    args = (antpos, 150e6, e2t, crd, I, bm)
    v = vis_gpu(*args, precision=precision, method=method)
    ref = oracle_same_inputs(args, precision)
    if nsrc == 0:
        np.testing.assert_equal(v, 0)
        return
    assert rel_frobenius(v, ref).max() <= TOL[(method, precision)]


@pytest.mark.parametrize("method,precision", METHODS)
def test_all_below_horizon(method, precision):
    rng = np.random.default_rng(5)
    crd = synth.sphere_sources(500, rng)
    crd[2] = -np.abs(crd[2]) - 1e-3
    v = vis_gpu(rng.normal(0, 30, (9, 3)), 150e6, np.array([np.identity(3)] * 2), crd,
                np.ones(500), np.ones((9, 7, 7)), precision=precision, method=method)
    np.testing.assert_equal(v, 0)


@pytest.mark.parametrize("method,precision", METHODS)
def test_multifreq_equals_per_frequency_calls(method, precision):
    cfg = synth.config_array(seed=3, nant=40, nsrc=3000, ntimes=3, nfreq=4, fmin=100e6,
                             fmax=200e6, P=31)
    bms = synth.beams_for(cfg, dtype=np.float64)
    multi = vis_gpu_multifreq(cfg["antpos"], cfg["freqs"], cfg["eq2tops"], cfg["crd_eq"],
                              cfg["I_sky"], bms, precision=precision, method=method)
    for f in range(len(cfg["freqs"])):
        single = vis_gpu(cfg["antpos"], cfg["freqs"][f], cfg["eq2tops"], cfg["crd_eq"],
                         cfg["I_sky"], bms[f], precision=precision, method=method)
        np.testing.assert_array_equal(multi[f], single)


@pytest.mark.parametrize("method,precision", METHODS)
def test_deterministic(method, precision):
    args, _ = load("random_inputs")
    a = vis_gpu(*args, precision=precision, method=method)
    b = vis_gpu(*args, precision=precision, method=method)
    np.testing.assert_array_equal(a, b)


def test_fp16_form_scales_each_slice():
    # the FP16 + FP8 form scales each (time, frequency) slice by its own
    # power of two: skies of very different brightness per channel (the beam
    # differs by 2^40 between channels) keep the same relative accuracy
    cfg = synth.config_array(seed=8, nant=60, nsrc=4000, ntimes=2, nfreq=3, fmin=100e6,
                             fmax=200e6, P=31)
    bms = synth.beams_for(cfg, dtype=np.float64)
    bms *= np.array([1e-6, 1.0, 1e6])[:, None, None, None]
    I = cfg["I_sky"] * 1e3
    v = vis_gpu_multifreq(cfg["antpos"], cfg["freqs"], cfg["eq2tops"], cfg["crd_eq"], I, bms,
                          precision=1, method="tc_fp16")
    for f in range(3):
        ref = oracle_same_inputs((cfg["antpos"], cfg["freqs"][f], cfg["eq2tops"], cfg["crd_eq"],
                                  I, bms[f]), 1)
        assert rel_frobenius(v[f], ref).max() <= 1e-4, f


@pytest.mark.parametrize("method", ["tc", "tc_fp16"])
@pytest.mark.parametrize("stages", [2, 3, 4])
def test_launch_shapes_agree(method, stages):
    # the tuning knobs change how the work is laid out on the SM, not the
    # arithmetic: every shape gives the default's result bit for bit
    from hera_gpu_gb300 import _native
    cfg = synth.config_array(seed=9, nant=300, nsrc=6000, ntimes=2, nfreq=2, fmin=100e6,
                             fmax=200e6, P=31)
    bms = synth.beams_for(cfg, dtype=np.float32)
    args = (cfg["antpos"], cfg["freqs"], cfg["eq2tops"], cfg["crd_eq"], cfg["I_sky"], bms)
    ctx = _native.Context(0)
    ref = vis_gpu_multifreq(*args, precision=1, method=method, context=ctx)
    ctx.set_tuning(stages=stages)
    got = vis_gpu_multifreq(*args, precision=1, method=method, context=ctx)
    np.testing.assert_array_equal(got, ref)


def test_sync_covers_a_call_on_the_callers_stream():
    # hv_vis_multifreq_device on a stream of the caller's, then hv_sync on
    # the context: the output is complete when hv_sync returns, without the
    # caller synchronising its own stream (the output starts as NaN, and the
    # call is long enough to still be running otherwise)
    import torch
    from hera_gpu_gb300 import _native
    cfg = synth.config_array(seed=4, nant=300, nsrc=200_000, ntimes=4, nfreq=8, fmin=100e6,
                             fmax=200e6, P=31)
    bms = synth.beams_for(cfg, dtype=np.float32)
    host = {k: np.ascontiguousarray(cfg[k], dtype=np.float32)
            for k in ("antpos", "eq2tops", "crd_eq", "I_sky")}
    dev = torch.device("cuda", 0)
    d = {k: torch.from_numpy(v).to(dev) for k, v in host.items()}
    d_bm = torch.from_numpy(bms).to(dev)
    ctx = _native.Context(0)
    ref = vis_gpu_multifreq(host["antpos"], cfg["freqs"], host["eq2tops"], host["crd_eq"],
                            host["I_sky"], bms, precision=1, method="tc", context=ctx)
    out = torch.full(ref.shape, float("nan"), dtype=torch.complex64, device=dev)
    stream = torch.cuda.Stream(dev)
    torch.cuda.synchronize(dev)
    ctx.vis_multifreq_device(1, "tc", d["antpos"].data_ptr(), 300, cfg["freqs"],
                             d["eq2tops"].data_ptr(), 4, d["crd_eq"].data_ptr(),
                             d["I_sky"].data_ptr(), 200_000, d_bm.data_ptr(), 31, out.data_ptr(),
                             stream.cuda_stream)
    ctx.sync()
    got = out.cpu().numpy()   # a copy on the default stream, not ordered after `stream`
    np.testing.assert_array_equal(got, ref)
