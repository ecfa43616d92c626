"""Outputs of the reference's own vis_gpu for the fixtures in this folder.

Runs the unmodified ``vis_gpu`` of hera_gpu/vis.py:144-262 -- its host loop,
and its InterpolateBeam / MeasEq kernels compiled for the host -- on the CPU
through oracle/vis_ref.py, at precision 1 and 2:

* on the inputs of small_config.npz, random_inputs.npz and edge_inputs.npz
  (whose vis_cpu outputs make_golden.py stored), so the reference's GPU
  function and its CPU test oracle are pinned on the same inputs;
* on a ragged case, 1003 sources, of which the reference sums the first
  1000 (vis.py:176-177), with an even 30-pixel beam.

Writes vis_gpu_reference.npz: per case, ``<case>_p1`` / ``<case>_p2`` (the
outputs) and ``<case>_nsrc_used``; the ragged case's inputs as
``ragged_<argument>``.

Usage (needs the reference sources; the fixture is committed):

    python tests/golden/make_vis_gpu_golden.py /path/to/reference
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

ARGS = ("antpos", "freq", "eq2tops", "crd_eq", "I_sky", "bm_cube")


def ragged_inputs():
    from hera_gpu_gb300 import synth
    rng = np.random.default_rng(7)
    nant, nsrc, ntimes, P = 5, 1003, 3, 30
    e2t = np.stack([np.linalg.qr(rng.normal(size=(3, 3)))[0] for _ in range(ntimes)])
    crd = synth.sphere_sources(nsrc, rng)
    # the three sources the reference drops: bright, near the first time's zenith
    near = e2t[0][2][:, None] + 0.05 * rng.normal(size=(3, 3))
    crd[:, -3:] = near / np.linalg.norm(near, axis=0)
    I_sky = rng.random(nsrc) * 2
    I_sky[-3:] = 5.0
    return dict(antpos=synth.disc_array(nant, 40.0, rng), freq=120e6, eq2tops=e2t,
                crd_eq=crd, I_sky=I_sky,
                bm_cube=synth.gaussian_beams(nant, P, rng.uniform(10.0, 20.0, nant)))


def main(ref_root):
    from oracle.vis_ref import reference_vis_gpu, sources_used

    cases = {}
    for name in ("small_config", "random_inputs", "edge_inputs"):
        z = np.load(os.path.join(HERE, name + ".npz"))
        cases[name] = {k: (float(z[k]) if k == "freq" else z[k]) for k in ARGS}
    cases["ragged"] = ragged_inputs()
    out = {}
    for name, a in cases.items():
        args = tuple(a[k] for k in ARGS)
        nant, nsrc = a["antpos"].shape[0], a["crd_eq"].shape[1]
        out[f"{name}_nsrc_used"] = sources_used(nant, nsrc)
        for p in (1, 2):
            out[f"{name}_p{p}"] = reference_vis_gpu(ref_root, *args, precision=p)
        if name == "ragged":
            out.update({f"ragged_{k}": v for k, v in a.items()})
        print(name, "sources used", out[f"{name}_nsrc_used"], "of", nsrc)
    np.savez_compressed(os.path.join(HERE, "vis_gpu_reference.npz"), **out)


if __name__ == "__main__":
    main(sys.argv[1])
