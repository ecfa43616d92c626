"""The seeded synthetic workloads (hera_gpu_gb300/synth.py) have the shapes,
sizes and value distributions their docstrings state -- the benchmark
configurations' -- and repeat per seed.  CPU only."""
import numpy as np
import pytest
from scipy.special import j1

from hera_gpu_gb300 import sky, synth


def test_config_small():
    c = synth.config_small(seed=0)
    assert c["antpos"].shape == (16, 3) and c["crd_eq"].shape == (3, 1000)
    assert c["eq2tops"].shape == (10, 3, 3) and c["bm_cubes"].shape == (1, 16, 31, 31)
    np.testing.assert_array_equal(c["freqs"], [150e6])
    assert np.all(np.hypot(c["antpos"][:, 0], c["antpos"][:, 1]) <= 50.0)
    assert np.all(c["antpos"][:, 2] == 0)
    assert c["I_sky"].min() >= 0.1 and c["I_sky"].max() <= 10.0
    np.testing.assert_allclose(np.linalg.norm(c["crd_eq"], axis=0), 1, atol=1e-12)
    # Gaussian beams are 1 at the zenith; the first LST is 0
    bm = c["bm_cubes"][0]
    np.testing.assert_allclose(bm[:, 15, 15], 1.0)
    e2t0 = sky.eq2top(0.0, np.radians(sky.HERA_LATITUDE_DEG))
    np.testing.assert_allclose(c["eq2tops"][0], e2t0)


def test_gaussian_beam_half_power_at_half_fwhm():
    P = 2001
    fwhm = np.array([10.0, 15.0])
    bm = synth.gaussian_beams(2, P, fwhm)
    g = np.linspace(-1, 1, P)
    th = np.degrees(np.arcsin(np.abs(g)))
    for a in range(2):
        row = bm[a, P // 2, P // 2:]             # along l from the zenith, falling
        half = np.interp(0.5, row[::-1], th[P // 2:][::-1])
        assert half == pytest.approx(fwhm[a] / 2, abs=1e-3)


def test_airy_beam_first_null():
    # (2 J1(x) / x)^2 is 1 at the zenith and 0 at its first null x = 3.8317,
    # i.e. sin(theta) = 1.2197 lambda / D
    freq, dish = 150e6, 14.0
    lam = synth.C_LIGHT / freq
    P = 4001
    bm = synth.airy_beams(1, P, freq, [dish])[0]
    g = np.linspace(-1, 1, P)
    assert bm[P // 2, P // 2] == 1.0
    s_null = 3.8317059702 * lam / (np.pi * dish)
    i = np.argmin(np.abs(g - s_null))
    assert bm[P // 2, i] < 1e-5
    x = np.pi * dish * g[i] / lam
    assert bm[P // 2, i] == pytest.approx((2 * j1(x) / x) ** 2, rel=1e-12)


def test_config_array_layout_and_fluxes():
    c = synth.config_array(seed=0, nant=350, nsrc=200_000, ntimes=3, nfreq=4, fmin=100e6,
                           fmax=200e6)
    pos = c["antpos"]
    assert pos.shape == (350, 3)
    # 14.6 m hex grid with 1 cm jitter: nearest neighbours 14.6 m apart
    d = np.hypot(pos[:, None, 0] - pos[None, :, 0], pos[:, None, 1] - pos[None, :, 1])
    np.fill_diagonal(d, np.inf)
    np.testing.assert_allclose(d.min(axis=1), 14.6, atol=0.06)
    assert np.std(pos[:, 2]) == pytest.approx(0.01, rel=0.2)
    np.testing.assert_allclose(c["freqs"], np.linspace(100e6, 200e6, 4))
    assert np.all(np.abs(c["dish"] / 14.0 - 1) <= 0.02)
    # power law dN/dS ~ S^-2 on [0.05, 50]: CDF (1/lo - 1/S) / (1/lo - 1/hi)
    S = c["I_sky"]
    assert S.min() >= 0.05 and S.max() <= 50.0
    for s in (0.1, 0.5, 5.0):
        cdf = (1 / 0.05 - 1 / s) / (1 / 0.05 - 1 / 50.0)
        assert np.mean(S <= s) == pytest.approx(cdf, abs=0.005)
    # sources uniform on the sphere: half above any plane through the origin
    z = c["crd_eq"][2]
    assert np.mean(z > 0) == pytest.approx(0.5, abs=0.005)
    assert np.mean(np.abs(z) < 0.5) == pytest.approx(0.5, abs=0.005)


def test_config_batch_sizes_and_sims():
    sims = synth.config_batch(seed=0, nsims=256)
    assert len(sims) == 256
    for s in sims:
        assert 16 <= s["nant"] <= 350 and 1000 <= s["nsrc"] <= 200_000
        assert 1 <= s["ntimes"] <= 60 and 1 <= s["nfreq"] <= 16 and s["P"] in (31, 63)
    # log-uniform: about half below the geometric mean
    nant = np.array([s["nant"] for s in sims])
    assert np.mean(nant < np.sqrt(16 * 350)) == pytest.approx(0.5, abs=0.1)
    spec = dict(sims[0], nsrc=500, ntimes=2, nfreq=3, P=31)
    sim = synth.make_sim(spec)
    assert sim["antpos"].shape == (spec["nant"], 3) and sim["antpos"].dtype == np.float32
    assert sim["bm_cubes"].shape == (3, spec["nant"], 31, 31)
    np.testing.assert_allclose(sim["freqs"], [100e6, 150e6, 200e6])
    assert sim["eq2tops"].shape == (2, 3, 3) and sim["crd_eq"].shape == (3, 500)


def test_generators_repeat_per_seed():
    a, b = synth.config_small(seed=4), synth.config_small(seed=4)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
    c = synth.config_small(seed=5)
    assert not np.array_equal(a["antpos"], c["antpos"])
    spec = synth.config_batch(seed=1, nsims=1)[0]
    spec.update(nsrc=100, ntimes=1, nfreq=1, P=31)
    s1, s2 = synth.make_sim(spec), synth.make_sim(spec)
    for k in s1:
        np.testing.assert_array_equal(s1[k], s2[k])
