"""Omnical redundant calibration (hera_gpu.redcal.omnical, redcal.py:358-743).

CPU: the oracle restatement against the reference's own known answers
(hera_gpu/tests/test_redcal.py:56-101: already-calibrated data stays put,
gains of 1.1 on unit data converge), against the reference's own omnical
run on the CPU (fixtures in tests/golden/, made by make_omnical_golden.py),
and against properties of the solution (a noiseless redundant problem is
solved to its data).  GPU: the library's
kernel through the drop-in ``omnical`` -- the same known answers and
fixtures, then parity with the oracle on seeded redundant arrays at both precisions, over
the launch shapes the kernel plans (one panel of baselines with the data in
shared memory; two and four panels with the data read from global memory),
and the edge cases
(no problems, maxiter 0, flagged baselines, bad indices, determinism and
independence of the problems from each other).
"""
import os

import numpy as np
import pytest

from hera_gpu_gb300 import synth
from oracle import omnical_oracle, redundant_problem

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FIXTURES = sorted(f[len("omnical_"):-len(".npz")] for f in os.listdir(GOLDEN)
                  if f.startswith("omnical_") and f.endswith(".npz"))


def load_fixture(name):
    """Inputs, schedule and the reference's own outputs (the reference's
    omnical run on the CPU, tests/golden/make_omnical_golden.py)."""
    z = np.load(os.path.join(GOLDEN, f"omnical_{name}.npz"))
    kw = {k: z[k].item() for k in ("conv_crit", "maxiter", "check_every", "check_after", "gain")
          if k in z}
    ref = {k[len("out_"):]: z[k] for k in z.files if k.startswith("out_")}
    return z, int(z["precision"]), kw, ref


def check_against_reference(got, ref, z, precision, gain_tol):
    """gains / ubls within gain_tol of their scale; chisq where the stopping
    iteration agrees; the stopping iteration itself, except where the
    criterion sits at the float64 rounding floor of the convergence measure
    (conv_crit 1e-12), where any summation order may stop a check earlier or
    later -- there the solutions must reproduce noiseless data as tightly as
    the reference's (test_redcal.py:118-125 asks for 10 decimals)."""
    same = got["iters"] == ref["iters"]
    floor = "conv_crit" in z.files and float(z["conv_crit"]) <= 1e-12
    if not floor:
        assert same.mean() >= (0.99 if precision == 2 else 0.9), (got["iters"], ref["iters"])
    for k in ("gains", "ubls"):
        np.testing.assert_allclose(got[k], ref[k], rtol=0,
                                   atol=gain_tol * np.nanmax(np.abs(ref[k])))
    # chi^2 to within rounding of the data's own energy sum |data|^2 w
    energy = np.sum(np.abs(z["data"].astype(np.complex128)) ** 2 * z["wgts"], axis=1)
    np.testing.assert_allclose(got["chisq"][same], ref["chisq"][same],
                               rtol=1e-6 if precision == 2 else 5e-3,
                               atol=(1e-13 if precision == 2 else 1e-6) * energy.max())
    if floor:
        ggu = z["ggu"].astype(np.int64)
        model = got["gains"][:, ggu[:, 0]] * np.conj(got["gains"][:, ggu[:, 1]]) * \
            got["ubls"][:, ggu[:, 2]]
        assert np.abs(model - z["data"]).max() <= 1e-10 * np.abs(z["data"]).max()

NANTS = 16


def linear_ggu(nants):
    """The reference's test layout (test_redcal.py:62-63)."""
    return synth.linear_redundant_layout(nants)[0]


hex_ggu = synth.hex_redundant_layout
make_problem = synth.redundant_data


# ---------------------------------------------------------------- CPU: oracle

def test_oracle_already_correct():
    # test_redcal.py:64-82 (the reference's assert_allclose(x, 1, 4) has rtol 4)
    nb = NANTS * (NANTS - 1) // 2
    for precision in (1, 2):
        info = omnical_oracle(linear_ggu(NANTS), np.ones((8, NANTS)), np.ones((8, 15)),
                              np.ones((8, nb)), np.ones((8, nb)), 1e-4, 100, 2, 1,
                              precision=precision)
        np.testing.assert_allclose(info["gains"], 1, 4)
        np.testing.assert_allclose(info["ubls"], 1, 4)
        np.testing.assert_allclose(info["chisq"], 0, 4)
        np.testing.assert_allclose(info["iters"], 1, 4)
        np.testing.assert_allclose(info["conv"], 0, 4)
        # and exactly: one step changes nothing, so the first check stops it
        assert np.all(info["gains"] == 1) and np.all(info["conv"] == 0)
        assert np.all(info["iters"] == 0) and np.all(info["chisq"] == 0)


def test_oracle_calibrate():
    # test_redcal.py:83-101
    nb = NANTS * (NANTS - 1) // 2
    for precision in (1, 2):
        crit = 1e-3 ** precision
        info = omnical_oracle(linear_ggu(NANTS), 1.1 * np.ones((8, NANTS)), np.ones((8, 15)),
                              np.ones((8, nb)), np.ones((8, nb)), crit, 100, 2, 1,
                              precision=precision)
        np.testing.assert_allclose(info["gains"], 1, 4)
        np.testing.assert_allclose(info["ubls"], 1, 4)
        np.testing.assert_allclose(info["chisq"], 0, atol=10)
        np.testing.assert_array_less(1, info["iters"])
        np.testing.assert_array_less(info["conv"], crit)


def test_oracle_solves_noiseless_redundant_data():
    ggu, nubls = hex_ggu(19)
    g0, u0, d, w = make_problem(ggu, nubls, 6, seed=3)
    info = omnical_oracle(ggu, g0, u0, d, w, 1e-12, 500, 4, 1)
    gi, gj, uk = (ggu[:, c].astype(np.int64) for c in range(3))
    model = info["gains"][:, gi] * np.conj(info["gains"][:, gj]) * info["ubls"][:, uk]
    assert np.max(np.abs(model - d)) < 1e-6
    assert np.all(info["chisq"] < 1e-10) and np.all(info["iters"] > 4)


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_matches_the_reference_omnical(name):
    # the oracle against the reference's own omnical on the same inputs
    z, precision, kw, ref = load_fixture(name)
    got = omnical_oracle(z["ggu"], z["gains"], z["ubls"], z["data"], z["wgts"],
                         precision=precision, **kw)
    check_against_reference(got, ref, z, precision, 1e-12 if precision == 2 else 2e-4)


def test_redundant_problem_helper_is_consistent():
    ggu, g, u, d, w = redundant_problem(12, 3, seed=2)
    gi, gj, uk = (ggu[:, c].astype(np.int64) for c in range(3))
    np.testing.assert_allclose(g[:, gi] * np.conj(g[:, gj]) * u[:, uk], d)


def test_hex_layout_is_redundant():
    ggu, nubls = hex_ggu(37)
    assert len(ggu) == 37 * 36 // 2 and nubls < len(ggu)
    assert ggu[:, 2].max() == nubls - 1


# ---------------------------------------------------------------- GPU

gpu = pytest.mark.gpu


@gpu
def test_already_correct():
    from hera_gpu_gb300 import omnical
    nubls, nbls, ndata = 15, NANTS * (NANTS - 1) // 2, 2048
    for precision in (1, 2):
        gains = np.ones((ndata, NANTS), dtype=np.complex64)
        ubls = np.ones((ndata, nubls), dtype=np.complex64)
        data = np.ones((ndata, nbls), dtype=np.complex64)
        wgts = np.ones((ndata, nbls), dtype=np.float32)
        info = omnical(linear_ggu(NANTS), gains, ubls, data, wgts, 1e-4, 100, 2, 1,
                       precision=precision)
        np.testing.assert_allclose(info["gains"], 1, 4)
        np.testing.assert_allclose(info["ubls"], 1, 4)
        np.testing.assert_allclose(info["chisq"], 0, 4)
        np.testing.assert_allclose(info["iters"], 1, 4)
        np.testing.assert_allclose(info["conv"], 0, 4)
        ct = np.complex64 if precision == 1 else np.complex128
        assert info["gains"].dtype == ct and info["ubls"].dtype == ct
        assert info["chisq"].dtype == np.dtype(ct).type(0).real.dtype
        assert info["iters"].dtype == np.uint32
        assert np.all(info["gains"] == 1) and np.all(info["conv"] == 0)
        assert np.all(gains == 1)     # inputs untouched


@gpu
def test_calibrate():
    from hera_gpu_gb300 import omnical
    nubls, nbls, ndata = 15, NANTS * (NANTS - 1) // 2, 2048
    for precision in (1, 2):
        gains = 1.1 * np.ones((ndata, NANTS), dtype=np.complex64)
        ubls = np.ones((ndata, nubls), dtype=np.complex64)
        data = np.ones((ndata, nbls), dtype=np.complex64)
        wgts = np.ones((ndata, nbls), dtype=np.float32)
        crit = 1e-3 ** precision
        info = omnical(linear_ggu(NANTS), gains, ubls, data, wgts, crit, 100, 2, 1,
                       precision=precision)
        np.testing.assert_allclose(info["gains"], 1, 4)
        np.testing.assert_allclose(info["ubls"], 1, 4)
        np.testing.assert_allclose(info["chisq"], 0, atol=10)
        np.testing.assert_array_less(1, info["iters"])
        np.testing.assert_array_less(info["conv"], crit)
        ref = omnical_oracle(linear_ggu(NANTS), gains[:4], ubls[:4], data[:4], wgts[:4], crit,
                             100, 2, 1, precision=precision)
        assert np.all(info["iters"] == ref["iters"][0])
        tol = 1e-5 if precision == 1 else 1e-12
        np.testing.assert_allclose(info["gains"], np.broadcast_to(ref["gains"][0], info["gains"].shape),
                                   rtol=tol, atol=tol)


def _parity(ggu, nubls, ndata, precision, seed, noise, crit, maxiter=200, check_every=4,
            check_after=1, gain=0.3, flag=0.0, allow_empty=False):
    from hera_gpu_gb300 import omnical
    g0, u0, d, w = make_problem(ggu, nubls, ndata, seed, noise=noise)
    if flag:
        w[np.random.default_rng(seed + 1).random(w.shape) < flag] = 0.0
        if not allow_empty:
            # keep one baseline of every unique baseline and of every antenna
            for k in range(nubls):
                w[:, np.flatnonzero(ggu[:, 2] == k)[0]] = 1.0
            for a in range(int(ggu[:, :2].max()) + 1):
                w[:, np.flatnonzero((ggu[:, 0] == a) | (ggu[:, 1] == a))[0]] = 1.0
    ct, rt = (np.complex64, np.float32) if precision == 1 else (np.complex128, np.float64)
    g0, u0, d, w = g0.astype(ct), u0.astype(ct), d.astype(ct), w.astype(rt)
    got = omnical(ggu, g0, u0, d, w, crit, maxiter, check_every, check_after, gain,
                  precision=precision)
    ref = omnical_oracle(ggu, g0, u0, d, w, crit, maxiter, check_every, check_after, gain,
                         precision=precision)
    same = got["iters"] == ref["iters"]
    if precision == 2:
        # float64 against float64, sums in another order
        assert same.mean() >= 0.99, (got["iters"], ref["iters"])
        tol = 1e-9
    else:
        # float32 against float64: a problem near its criterion may stop one
        # check earlier or later, a change below the criterion
        assert same.mean() >= 0.9, (got["iters"], ref["iters"])
        tol = 2e-4
    # NaN where the reference gives NaN (a unique baseline or an antenna
    # with every baseline flagged: a 0 / 0 weight), equal elsewhere
    scale = np.nanmax(np.abs(ref["gains"]))
    np.testing.assert_allclose(got["gains"], ref["gains"], rtol=0, atol=tol * scale)
    np.testing.assert_allclose(got["ubls"], ref["ubls"], rtol=0,
                               atol=tol * np.nanmax(np.abs(ref["ubls"])))
    cs = np.maximum(np.abs(ref["chisq"]), 1e-30)
    np.testing.assert_allclose(got["chisq"][same], ref["chisq"][same],
                               rtol=1e-6 if precision == 2 else 5e-3,
                               atol=(1e-12 if precision == 2 else 1e-5) * np.nanmax(cs))
    return got, ref


@gpu
@pytest.mark.parametrize("name", FIXTURES)
def test_omnical_matches_the_reference_omnical(name):
    # the library against the reference's own omnical on the same inputs
    from hera_gpu_gb300 import omnical
    z, precision, kw, ref = load_fixture(name)
    got = omnical(z["ggu"], z["gains"], z["ubls"], z["data"], z["wgts"], precision=precision,
                  **kw)
    check_against_reference(got, ref, z, precision, 1e-9 if precision == 2 else 2e-4)


@gpu
@pytest.mark.parametrize("precision", [1, 2])
def test_parity_linear16(precision):
    _parity(linear_ggu(16), 15, 300, precision, seed=11, noise=0.01,
            crit=1e-5 if precision == 1 else 1e-10)


@gpu
@pytest.mark.parametrize("precision", [1, 2])
@pytest.mark.parametrize("nants", [7, 37, 61])
def test_parity_hex(precision, nants):
    ggu, nubls = hex_ggu(nants)
    _parity(ggu, nubls, 96, precision, seed=nants, noise=0.02,
            crit=1e-5 if precision == 1 else 1e-10)


@gpu
@pytest.mark.parametrize("precision", [1, 2])
@pytest.mark.parametrize("nants", [128, 200])
def test_parity_large_arrays(precision, nants):
    # 8128 baselines: float32 in one panel with data and weights in shared
    # memory, float64 in two panels; 19900 baselines: two (float32) and four
    # (float64) panels
    _parity(linear_ggu(nants), nants - 1, 8, precision, seed=5, noise=0.02,
            crit=1e-5 if precision == 1 else 1e-10, maxiter=60)


@gpu
@pytest.mark.parametrize("check_every,check_after,gain", [(2, 1, 0.3), (6, 30, 0.5), (4, 9, 0.1),
                                                          (3, 1, 0.45)])
def test_parity_schedules(check_every, check_after, gain):
    ggu, nubls = hex_ggu(19)
    _parity(ggu, nubls, 64, 2, seed=check_every * 7 + check_after, noise=0.01, crit=1e-10,
            maxiter=120, check_every=check_every, check_after=check_after, gain=gain)


@gpu
@pytest.mark.parametrize("precision", [1, 2])
def test_parity_flagged_baselines(precision):
    ggu, nubls = hex_ggu(37)
    got, _ = _parity(ggu, nubls, 64, precision, seed=9, noise=0.01,
                     crit=1e-5 if precision == 1 else 1e-10, flag=0.2)
    assert np.all(np.isfinite(got["gains"]))


@gpu
def test_fully_flagged_unique_baseline_gives_nan_as_the_reference():
    ggu, nubls = hex_ggu(37)
    got, ref = _parity(ggu, nubls, 64, 2, seed=9, noise=0.01, crit=1e-10, flag=0.1,
                       allow_empty=True)
    assert np.isnan(ref["gains"]).any()
    np.testing.assert_array_equal(np.isnan(got["gains"]), np.isnan(ref["gains"]))


@gpu
def test_maxiter_limits_and_zero():
    from hera_gpu_gb300 import omnical
    ggu, nubls = hex_ggu(19)
    g0, u0, d, w = make_problem(ggu, nubls, 8, seed=4, noise=0.01)
    for maxiter in (0, 1, 3):
        got = omnical(ggu, g0, u0, d, w, 1e-14, maxiter, 4, 1, precision=2)
        ref = omnical_oracle(ggu, g0, u0, d, w, 1e-14, maxiter, 4, 1, precision=2)
        np.testing.assert_array_equal(got["iters"], ref["iters"])
        np.testing.assert_allclose(got["gains"], ref["gains"], rtol=0, atol=1e-12)
        np.testing.assert_allclose(got["chisq"], ref["chisq"], rtol=1e-9)
        if maxiter == 0:
            np.testing.assert_array_equal(got["gains"], g0)
            assert np.all(got["conv"] == 0) and np.all(got["iters"] == 0)


@gpu
def test_no_problems_and_bad_indices():
    from hera_gpu_gb300 import omnical
    from hera_gpu_gb300._native import HeraVisError
    ggu = linear_ggu(8)
    info = omnical(ggu, np.ones((0, 8)), np.ones((0, 7)), np.ones((0, 28)), np.ones((0, 28)))
    assert info["gains"].shape == (0, 8) and info["chisq"].shape == (0,)
    bad = ggu.copy()
    bad[5, 2] = 7     # unique baseline 7 of 7
    with pytest.raises(HeraVisError):
        omnical(bad, np.ones((2, 8)), np.ones((2, 7)), np.ones((2, 28)), np.ones((2, 28)))
    with pytest.raises(AssertionError):
        omnical(ggu, np.ones((2, 8)), np.ones((2, 7)), np.ones((2, 28)), np.ones((2, 28)),
                check_every=1)


@gpu
@pytest.mark.parametrize("precision", [1, 2])
def test_deterministic_and_independent(precision):
    from hera_gpu_gb300 import omnical
    ggu, nubls = hex_ggu(37)
    g0, u0, d, w = make_problem(ggu, nubls, 200, seed=21, noise=0.02)
    crit = 1e-5 if precision == 1 else 1e-10
    a = omnical(ggu, g0, u0, d, w, crit, 100, precision=precision)
    b = omnical(ggu, g0, u0, d, w, crit, 100, precision=precision)
    c = omnical(ggu, g0[37:41], u0[37:41], d[37:41], w[37:41], crit, 100, precision=precision)
    for k in ("gains", "ubls", "chisq", "iters", "conv"):
        np.testing.assert_array_equal(a[k], b[k])
        np.testing.assert_array_equal(a[k][37:41], c[k])
