"""Generate the omnical fixtures in this folder from the reference itself.

Runs the reference's own ``omnical`` (hera_gpu/redcal.py:358-743: its host
loop and its CUDA kernels, executed on the CPU by oracle/redcal_ref.py) on
seeded redundant-calibration problems and stores inputs and outputs as
``omnical_*.npz``:

* ``kat_calibrate_p1``, ``kat_calibrate_p2``: the known-answer case of the
  reference's test_calibrate (test_redcal.py:83-101): gains of 1.1 on unit
  data of a 16-antenna linear array;
* ``hex19_p1``, ``hex19_p2``: a 19-antenna hex array, 1% noise, the
  reference's default schedule;
* ``wrap16_p2``: noiseless data of a 16-antenna linear array with 1% gain
  scatter and the schedule of the reference's test_wrap
  (test_redcal.py:106-116: gain 0.5, check_every 6, check_after 30,
  conv_crit 1e-12, maxiter 500);
* ``hex37_flagged_p2``: a 37-antenna hex array with 10% of the baselines at
  zero weight (every antenna and unique baseline keeping one);
* ``linear64_p1``: 64 antennas (2016 baselines).

Usage (needs the reference sources; the fixtures are committed, so the GPU
machine never runs this):

    python tests/golden/make_omnical_golden.py /path/to/reference
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from hera_gpu_gb300 import synth  # noqa: E402
from oracle.redcal_ref import reference_omnical  # noqa: E402


def case(ggu, nubls, ndata, seed, precision, noise=0.01, scatter=0.05, flag=0.0, unit=False):
    ct, rt = (np.complex64, np.float32) if precision == 1 else (np.complex128, np.float64)
    if unit:
        nants = int(ggu[:, :2].max()) + 1
        g0 = 1.1 * np.ones((ndata, nants))
        u0 = np.ones((ndata, nubls))
        d = np.ones((ndata, len(ggu)))
        w = np.ones(d.shape)
    else:
        g0, u0, d, w = synth.redundant_data(ggu, nubls, ndata, seed=seed, noise=noise,
                                            scatter=scatter)
    if flag:
        w[np.random.default_rng(seed + 1).random(w.shape) < flag] = 0.0
        for k in range(nubls):
            w[:, np.flatnonzero(ggu[:, 2] == k)[0]] = 1.0
        for a in range(int(ggu[:, :2].max()) + 1):
            w[:, np.flatnonzero((ggu[:, 0] == a) | (ggu[:, 1] == a))[0]] = 1.0
    return ggu, g0.astype(ct), u0.astype(ct), d.astype(ct), w.astype(rt)


def main(ref_root):
    lin16, n16 = synth.linear_redundant_layout(16)
    hex19, n19 = synth.hex_redundant_layout(19)
    hex37, n37 = synth.hex_redundant_layout(37)
    lin64, n64 = synth.linear_redundant_layout(64)
    cases = {
        "kat_calibrate_p1": (case(lin16, n16, 8, 0, 1, unit=True), 1,
                             dict(conv_crit=1e-3, maxiter=100, check_every=2, check_after=1)),
        "kat_calibrate_p2": (case(lin16, n16, 8, 0, 2, unit=True), 2,
                             dict(conv_crit=1e-6, maxiter=100, check_every=2, check_after=1)),
        "hex19_p1": (case(hex19, n19, 32, 4, 1), 1, dict(conv_crit=1e-5, maxiter=150)),
        "hex19_p2": (case(hex19, n19, 32, 4, 2), 2, dict(conv_crit=1e-10, maxiter=150)),
        "wrap16_p2": (case(lin16, n16, 16, 6, 2, noise=0.0, scatter=0.01), 2,
                      dict(conv_crit=1e-12, maxiter=500, check_every=6, check_after=30, gain=0.5)),
        "hex37_flagged_p2": (case(hex37, n37, 16, 9, 2, flag=0.1), 2,
                             dict(conv_crit=1e-10, maxiter=200)),
        "linear64_p1": (case(lin64, n64, 8, 5, 1, noise=0.02), 1,
                        dict(conv_crit=1e-5, maxiter=80)),
    }
    for name, ((ggu, g0, u0, d, w), precision, kw) in cases.items():
        out = reference_omnical(ref_root, ggu, g0, u0, d, w, precision=precision, **kw)
        np.savez_compressed(
            os.path.join(HERE, f"omnical_{name}.npz"), ggu=ggu, gains=g0, ubls=u0, data=d,
            wgts=w, precision=precision, **{k: np.array(v) for k, v in kw.items()},
            out_gains=out["gains"], out_ubls=out["ubls"], out_chisq=out["chisq"],
            out_iters=out["iters"], out_conv=out["conv"])
        print(name, "iters", np.unique(out["iters"]))


if __name__ == "__main__":
    main(sys.argv[1])
