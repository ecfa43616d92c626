"""Seeded synthetic workloads with the shapes and value distributions of the
benchmark configurations (there is no network and no observed data here).

Each generator returns plain numpy arrays in the argument order of
``vis_gpu(antpos, freq, eq2tops, crd_eq, I_sky, bm_cube)``:

* ``antpos``  (nant, 3) metres, topocentric (E, N, U);
* ``freqs``   (nfreq,) Hz;
* ``eq2tops`` (ntimes, 3, 3) rotations for LSTs spanning the stated hours at
  latitude -30.72 deg (:mod:`hera_gpu_gb300.sky`);
* ``crd_eq``  (3, nsrc) equatorial unit vectors, uniform on the sphere;
* ``I_sky``   (nsrc,) Jy;
* ``bm_cubes`` (nfreq, nant, P, P) beam power on the (l, m) grid
  ``linspace(-1, 1, P)`` (axis order ``[ant, m(y), l(x)]`` as the reference's
  ``bm_cube``).

and, for the Omnical solver, redundant array layouts (``ggu_indices``) and
seeded redundant-calibration problems (``redundant_data``).
"""
from __future__ import annotations

import numpy as np

from . import sky

C_LIGHT = 299792458.0


def disc_array(nant, radius_m, rng):
    r = radius_m * np.sqrt(rng.random(nant))
    th = 2 * np.pi * rng.random(nant)
    return np.stack([r * np.cos(th), r * np.sin(th), np.zeros(nant)], axis=1)


def hex_array(nant, spacing_m, jitter_m, rng):
    """``nant`` points of a hexagonal lattice nearest the origin (ties broken
    by angle), plus isotropic Gaussian position jitter."""
    k = int(np.ceil(np.sqrt(nant))) + 2
    i, j = np.meshgrid(np.arange(-k, k + 1), np.arange(-k, k + 1), indexing="ij")
    x = spacing_m * (i + 0.5 * j)
    y = spacing_m * (np.sqrt(3) / 2) * j
    x, y = x.ravel(), y.ravel()
    order = np.lexsort((np.arctan2(y, x), np.round(np.hypot(x, y), 6)))[:nant]
    pos = np.stack([x[order], y[order], np.zeros(nant)], axis=1)
    return pos + rng.normal(0.0, jitter_m, size=pos.shape)


def sphere_sources(nsrc, rng):
    z = rng.uniform(-1.0, 1.0, nsrc)
    phi = rng.uniform(0.0, 2 * np.pi, nsrc)
    r = np.sqrt(1.0 - z * z)
    return np.stack([r * np.cos(phi), r * np.sin(phi), z])


def loguniform_flux(nsrc, lo, hi, rng):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), nsrc))


def powerlaw_flux(nsrc, index, lo, hi, rng):
    """Fluxes with dN/dS ~ S**index on [lo, hi] (inverse-CDF sampling)."""
    a = index + 1.0
    u = rng.random(nsrc)
    if abs(a) < 1e-12:
        return lo * np.exp(u * np.log(hi / lo))
    return (lo ** a + u * (hi ** a - lo ** a)) ** (1.0 / a)


def _grid_sin_theta(P):
    g = np.linspace(-1.0, 1.0, P)
    m, l = np.meshgrid(g, g, indexing="ij")   # [y, x]
    return np.minimum(np.hypot(l, m), 1.0)


def gaussian_beams(nant, P, fwhm_deg):
    """Gaussian power beams in zenith angle, one FWHM per antenna."""
    th = np.arcsin(_grid_sin_theta(P))
    sig = np.radians(np.asarray(fwhm_deg, dtype=np.float64)) / (2 * np.sqrt(2 * np.log(2)))
    return np.exp(-0.5 * (th[None] / sig[:, None, None]) ** 2)


def airy_beams(nant, P, freq_hz, dish_m):
    """Airy power beams ``(2 J1(x) / x)**2``, ``x = pi D sin(theta) / lambda``,
    with one effective dish diameter per antenna."""
    from scipy.special import j1
    st = _grid_sin_theta(P)
    lam = C_LIGHT / float(freq_hz)
    d = np.asarray(dish_m, dtype=np.float64)
    x = np.pi * d[:, None, None] * st[None] / lam
    safe = np.where(x == 0, 1.0, x)
    return np.where(x == 0, 1.0, (2 * j1(safe) / safe) ** 2)


def config_small(seed=0):
    """16 antennas in a 100 m (diameter) disc, 1000 sources, 10 times, one
    150 MHz channel, Gaussian beams 31x31 with FWHM 10-15 deg."""
    rng = np.random.default_rng(seed)
    nant, nsrc, ntimes, P = 16, 1000, 10, 31
    antpos = disc_array(nant, 50.0, rng)
    crd_eq = sphere_sources(nsrc, rng)
    I_sky = loguniform_flux(nsrc, 0.1, 10.0, rng)
    fwhm = rng.uniform(10.0, 15.0, nant)
    bm = gaussian_beams(nant, P, fwhm)[None]
    lsts = sky.lst_grid(ntimes, 1.0)
    e2t = sky.eq2tops(lsts, np.radians(sky.HERA_LATITUDE_DEG))
    return dict(antpos=antpos, freqs=np.array([150e6]), eq2tops=e2t,
                crd_eq=crd_eq, I_sky=I_sky, bm_cubes=bm)


def config_array(seed=0, nant=350, nsrc=100_000, ntimes=60, nfreq=1,
                 fmin=150e6, fmax=150e6, P=63, hours=1.0):
    """Array-scale workload: ``nant`` on a 14.6 m hex grid with 1 cm jitter,
    sphere-uniform power-law sources (index -2, 0.05-50 Jy), Airy beams of a
    14 m dish (per-antenna diameter jitter of 2 %), ``nfreq`` channels evenly
    spaced on [fmin, fmax], ``ntimes`` LSTs over ``hours``."""
    rng = np.random.default_rng(seed)
    antpos = hex_array(nant, 14.6, 0.01, rng)
    crd_eq = sphere_sources(nsrc, rng)
    I_sky = powerlaw_flux(nsrc, -2.0, 0.05, 50.0, rng)
    dish = 14.0 * (1.0 + 0.02 * rng.uniform(-1.0, 1.0, nant))
    freqs = np.linspace(fmin, fmax, nfreq) if nfreq > 1 else np.array([fmin])
    lsts = sky.lst_grid(ntimes, hours)
    e2t = sky.eq2tops(lsts, np.radians(sky.HERA_LATITUDE_DEG))
    return dict(antpos=antpos, freqs=freqs, eq2tops=e2t, crd_eq=crd_eq,
                I_sky=I_sky, dish=dish, P=P)


def beams_for(cfg, dtype=np.float32, freqs=None):
    """Airy beam cubes (nfreq, nant, P, P) for an :func:`config_array` dict."""
    freqs = cfg["freqs"] if freqs is None else freqs
    out = np.empty((len(freqs), len(cfg["dish"]), cfg["P"], cfg["P"]), dtype=dtype)
    for i, f in enumerate(freqs):
        out[i] = airy_beams(len(cfg["dish"]), cfg["P"], f, cfg["dish"])
    return out


def config_batch(seed=0, nsims=256):
    """Size distribution of the batched form: per simulation nant
    log-uniform in [16, 350], nsrc log-uniform in [1e3, 2e5], ntimes uniform in
    [1, 60], nfreq uniform in [1, 16] over 100-200 MHz, beam P in {31, 63}.
    Returns a list of small dicts of sizes (arrays are made by
    :func:`make_sim`)."""
    rng = np.random.default_rng(seed)
    sims = []
    for i in range(nsims):
        sims.append(dict(
            seed=int(rng.integers(0, 2**31 - 1)),
            nant=int(np.round(np.exp(rng.uniform(np.log(16), np.log(350))))),
            nsrc=int(np.round(np.exp(rng.uniform(np.log(1e3), np.log(2e5))))),
            ntimes=int(rng.integers(1, 61)),
            nfreq=int(rng.integers(1, 17)),
            P=int(rng.choice([31, 63]))))
    return sims


def make_sim_arrays(spec, dtype=np.float32):
    """Everything of :func:`make_sim` but the beam cubes: the arrays, and the
    per-antenna dish diameters the Airy beams are made from."""
    rng = np.random.default_rng(spec["seed"])
    full = hex_array(350, 14.6, 0.01, rng)
    pick = np.sort(rng.choice(350, size=spec["nant"], replace=False))
    antpos = full[pick]
    crd_eq = sphere_sources(spec["nsrc"], rng)
    I_sky = powerlaw_flux(spec["nsrc"], -2.0, 0.05, 50.0, rng)
    nf = spec["nfreq"]
    freqs = np.linspace(100e6, 200e6, nf) if nf > 1 else np.array([150e6])
    dish = 14.0 * (1.0 + 0.02 * rng.uniform(-1.0, 1.0, spec["nant"]))
    lsts = sky.lst_grid(spec["ntimes"], 1.0, start_rad=rng.uniform(0, 2 * np.pi))
    e2t = sky.eq2tops(lsts, np.radians(sky.HERA_LATITUDE_DEG))
    return dict(antpos=antpos.astype(dtype), freqs=freqs, eq2tops=e2t.astype(dtype),
                crd_eq=crd_eq.astype(dtype), I_sky=I_sky.astype(dtype)), dish


def make_sim(spec, dtype=np.float32):
    """Arrays for one simulation of :func:`config_batch`: antennas on a random
    subset of the 350-element hex grid, sphere-uniform power-law sources,
    Airy beams, frequencies evenly spaced in 100-200 MHz."""
    sim, dish = make_sim_arrays(spec, dtype)
    bm = np.empty((len(sim["freqs"]), spec["nant"], spec["P"], spec["P"]), dtype=dtype)
    for i, f in enumerate(sim["freqs"]):
        bm[i] = airy_beams(spec["nant"], spec["P"], f, dish)
    sim["bm_cubes"] = bm
    return sim


# ---- redundant-calibration problems (omnical) ------------------------------

def linear_redundant_layout(nants):
    """Every pair i > j of a linear array of nants evenly spaced antennas,
    unique baseline i - j - 1 (the layout of hera_gpu's omnical tests,
    test_redcal.py:62-63): (ggu_indices (nbls, 3) uint32, nubls)."""
    ggu = np.array([(i, j, i - j - 1) for i in range(nants) for j in range(i)],
                   dtype=np.uint32).reshape(-1, 3)
    return ggu, max(nants - 1, 0)


def hex_redundant_layout(nants):
    """A 2-D redundant array: the nants points of a triangular lattice
    nearest its centre; every pair oriented so its separation vector is
    canonical (lexicographically positive), unique baselines numbered by
    distinct separation in pair order: (ggu_indices (nbls, 3) uint32, nubls)."""
    r = int(np.ceil(np.sqrt(nants))) + 2
    pts = [(a, b) for a in range(-r, r + 1) for b in range(-r, r + 1)]
    pts.sort(key=lambda p: (p[0] ** 2 + p[1] ** 2 + p[0] * p[1], p))
    pts = pts[:nants]
    ubl, out = {}, []
    for i in range(nants):
        for j in range(i):
            v = (pts[i][0] - pts[j][0], pts[i][1] - pts[j][1])
            a, b = i, j
            if v < (0, 0):
                v, a, b = (-v[0], -v[1]), j, i
            out.append((a, b, ubl.setdefault(v, len(ubl))))
    return np.array(out, dtype=np.uint32).reshape(-1, 3), len(ubl)


def redundant_data(ggu, nubls, ndata, seed=0, noise=0.0, scatter=0.05, perturb=0.02):
    """ndata redundant problems on the layout ggu: true gains 1 + scatter
    (complex normal), unit-variance complex unique baselines, data with
    complex noise of rms `noise` per component, unit weights, and a starting
    point -- gains perturbed by `perturb`, unique baselines averaged over
    their group from those gains.  Returns (gains0, ubls0, data, wgts), all
    complex128 / float64."""
    rng = np.random.default_rng(seed)
    nants = int(ggu[:, :2].max()) + 1 if len(ggu) else 0
    gi, gj, uk = (ggu[:, c].astype(np.int64) for c in range(3))
    g = 1 + scatter * (rng.normal(size=(ndata, nants)) + 1j * rng.normal(size=(ndata, nants)))
    u = rng.normal(size=(ndata, nubls)) + 1j * rng.normal(size=(ndata, nubls))
    d = g[:, gi] * np.conj(g[:, gj]) * u[:, uk]
    if noise:
        d = d + noise * (rng.normal(size=d.shape) + 1j * rng.normal(size=d.shape))
    w = np.ones(d.shape)
    g0 = g * (1 + perturb * (rng.normal(size=g.shape) + 1j * rng.normal(size=g.shape)))
    r = d / (g0[:, gi] * np.conj(g0[:, gj]))
    cnt = np.maximum(np.bincount(uk, minlength=nubls), 1)
    u0 = np.zeros((ndata, nubls), complex)
    for k in range(nubls):
        u0[:, k] = r[:, uk == k].sum(axis=1)
    return g0, u0 / cnt, d, w
