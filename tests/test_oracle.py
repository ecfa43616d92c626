"""The oracle against the reference's own outputs and known answers (CPU).

The fixtures under tests/golden/ were produced by running the reference's
``vis_cpu`` (hera_gpu/tests/test_vis_gpu.py:278-357; make_golden.py) and the
reference's ``vis_gpu`` itself -- its host loop and kernels, run on the CPU
(hera_gpu/vis.py:144-262; make_vis_gpu_golden.py) -- on the same inputs.
"""
import os

import numpy as np
import pytest
from scipy.interpolate import RectBivariateSpline

from oracle import bilinear_beam, rel_frobenius, vis_oracle
from oracle.vis_oracle import SPEED_OF_LIGHT, phasors
from vis_gpu_cases import VIS_GPU_CASES, load_vis_gpu_case

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = ["small_config", "random_inputs", "edge_inputs"]


def load(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    args = (d["antpos"], float(d["freq"]), d["eq2tops"], d["crd_eq"], d["I_sky"], d["bm_cube"])
    return args, d


@pytest.mark.parametrize("name", CASES)
def test_oracle_fp64_matches_reference(name):
    args, d = load(name)
    out = vis_oracle(*args, dtype=np.float64)
    assert out.shape == d["vis_p2"].shape
    # the reference's precision=2 run, to FP64 rounding
    assert rel_frobenius(out, d["vis_p2"]).max() < 1e-13
    np.testing.assert_allclose(out, d["vis_p2"], rtol=0, atol=1e-12 * np.abs(d["vis_p2"]).max())


@pytest.mark.parametrize("name", CASES)
def test_oracle_fp32_mode_matches_reference_fp32(name):
    args, d = load(name)
    out = vis_oracle(*args, dtype=np.float32)
    assert out.dtype == np.complex64
    assert rel_frobenius(out, d["vis_p1"]).max() < 1e-5


@pytest.mark.parametrize("P", [2, 5, 31])
def test_bilinear_matches_rectbivariatespline(P):
    rng = np.random.default_rng(P)
    beam = rng.random((P, P))
    x = rng.uniform(-1.3, 1.3, 4000)
    y = rng.uniform(-1.3, 1.3, 4000)
    x[:4] = [-1.0, 1.0, 0.0, 1.0]
    y[:4] = [1.0, -1.0, 0.0, 1.0]
    g = np.linspace(-1, 1, P)
    ref = RectBivariateSpline(g, g, beam, kx=1, ky=1)(y, x, grid=False)
    np.testing.assert_allclose(bilinear_beam(beam, x, y), ref, rtol=1e-12, atol=1e-14)


def test_hermitian_structure():
    args, d = load("small_config")
    out = vis_oracle(*args)
    np.testing.assert_array_equal(out, np.conj(np.transpose(out, (0, 2, 1))))
    assert np.all(np.diagonal(out, axis1=1, axis2=2).imag == 0)


# Known answers of the reference's test_values (test_vis_gpu.py:203-244),
# restated on the oracle.
NANT, NTIMES, BM_PIX, NPIX = 16, 10, 31, 12 * 16 ** 2


def kat_inputs():
    antpos = np.ones((NANT, 3))
    eq2tops = np.array([np.identity(3)] * NTIMES)
    crd_eq = np.zeros((3, NPIX))
    crd_eq[2] = 1
    return antpos, eq2tops, crd_eq, np.ones(NPIX), np.ones((NANT, BM_PIX, BM_PIX))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_kat_zero_sky_zero_beam_and_sum(dtype):
    antpos, eq2tops, crd_eq, I_sky, bm = kat_inputs()
    np.testing.assert_equal(vis_oracle(antpos, 1.0, eq2tops, crd_eq, I_sky * 0, bm, dtype), 0)
    np.testing.assert_equal(vis_oracle(antpos, 1.0, eq2tops, crd_eq, I_sky, bm * 0, dtype), 0)
    # The reference asks for decimal 22 (exact).  In FP64 the phase is
    # 2.1e-8 rad, cos() rounds to 1 - 2**-52 and the BLAS summation order of
    # the oracle leaves ~1.5e-16 relative; FP32 rounds every term to 1.
    decimal = 22 if dtype == np.float32 else 9
    np.testing.assert_almost_equal(vis_oracle(antpos, 1.0, eq2tops, crd_eq, I_sky, bm, dtype), NPIX, decimal)


def test_kat_two_sources():
    antpos, eq2tops, _, _, bm = kat_inputs()
    crd_eq = np.zeros((3, 2))
    crd_eq[2, 0] = 1
    crd_eq[1, 1] = np.sqrt(0.5)
    crd_eq[2, 1] = np.sqrt(0.5)
    v = vis_oracle(antpos, 1.0, eq2tops, crd_eq, np.ones(2), bm)
    np.testing.assert_almost_equal(v, 2, 2)


# Known answers of the reference's kernel tests, restated on the oracle's
# phasors (antennas at the origin, so v = A sqrt(I)).
def test_kat_beam_interpolation_flat_and_middle():
    # test_vis_gpu.py:31-65: a flat beam gives 1 above the horizon, 0 below
    flat = np.ones((8, 31, 31))
    crd = np.zeros((3, 128))
    crd[2] = 0.9
    args = (np.zeros((8, 3)), 150e6, np.identity(3))
    np.testing.assert_array_equal(phasors(*args, crd, np.ones(128), flat), 1)
    crd[2] = -0.9
    np.testing.assert_array_equal(phasors(*args, crd, np.ones(128), flat), 0)
    # test_vis_gpu.py:66-102: a beam of one centre pixel gives 1 at zenith,
    # 0 at 45 degrees off it
    middle = np.zeros((8, 31, 31))
    middle[:, 15, 15] = 1.0
    crd[:] = 0
    crd[2] = 1.0
    np.testing.assert_array_equal(phasors(*args, crd, np.ones(128), middle), 1)
    crd[1] = crd[2] = 0.5 ** 0.5
    np.testing.assert_array_equal(phasors(*args, crd, np.ones(128), middle), 0)


def test_kat_whole_cycle_phase():
    # test_vis_gpu.py:103-139: a delay of a whole number of cycles gives v = 1
    freq = 150e6
    antpos = np.zeros((2, 3))
    antpos[1, 2] = 10 * SPEED_OF_LIGHT / freq        # ten wavelengths up
    crd = np.array([[0.0], [0.0], [1.0]])
    v = phasors(antpos, freq, np.identity(3), crd, np.ones(1), np.ones((2, 31, 31)))
    np.testing.assert_allclose(v, 1, rtol=0, atol=1e-12)


def as_f32(x):
    return np.asarray(x).astype(np.float32).astype(np.float64)


@pytest.mark.parametrize("name", VIS_GPU_CASES)
def test_oracle_matches_the_reference_vis_gpu(name):
    used, _, out = load_vis_gpu_case(name)
    # FP64: the reference's vis_gpu and the oracle agree to rounding
    # (measured <= 3e-16, sources past the beam grid's edge included)
    assert rel_frobenius(out[2], vis_oracle(*used)).max() < 1e-13
    # FP32: the reference's own error, on the inputs as it sees them; its
    # delays come from an FP32 GEMM, so km baselines (edge_inputs) carry 3.5e-4
    a, f, e, s, i, b = used
    ref32 = vis_oracle(as_f32(a), f, as_f32(e), as_f32(s), as_f32(i), as_f32(b))
    bound = 1e-3 if name == "edge_inputs" else 1e-5
    assert rel_frobenius(out[1], ref32).max() < bound


def test_reference_vis_gpu_drops_the_remainder_sources():
    # vis.py:176-177: 1003 sources in 8 chunks of 125; the last 3 are not summed
    used, full, out = load_vis_gpu_case("ragged")
    assert used[3].shape[1] == 1000 and full[3].shape[1] == 1003
    assert rel_frobenius(out[2], vis_oracle(*full)).max() > 1e-4
