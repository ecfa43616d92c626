"""Generate the golden fixtures in this folder from the reference itself.

Runs the reference's own CPU implementation ``vis_cpu``
(``hera_gpu/tests/test_vis_gpu.py:278-357`` of the reference sources) on
seeded inputs and stores inputs and outputs as ``.npz``.  The reference test
module imports pycuda, scikit-cuda and astropy at module level
(test_vis_gpu.py:2-8, vis.py:1-4); none of them is needed by ``vis_cpu``, so
they are stubbed here (astropy's speed of light is 299 792 458 m/s).

Usage (needs the reference sources; the fixtures are committed, so the GPU
machine never runs this):

    python tests/golden/make_golden.py /path/to/reference
"""
from __future__ import annotations

import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def load_reference_vis_cpu(ref_root):
    for name in ["pycuda", "pycuda.autoinit", "pycuda.compiler", "pycuda.gpuarray",
                 "pycuda.driver", "skcuda", "skcuda.cublas", "astropy",
                 "astropy.constants"]:
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["astropy.constants"].c = types.SimpleNamespace(value=299792458.0)
    pkg = types.ModuleType("hera_gpu")
    pkg.__path__ = []
    vis = types.ModuleType("hera_gpu.vis")
    vis.vis_gpu = None
    pkg.vis = vis
    sys.modules["hera_gpu"] = pkg
    sys.modules["hera_gpu.vis"] = vis
    path = os.path.join(ref_root, "hera_gpu", "tests", "test_vis_gpu.py")
    spec = importlib.util.spec_from_file_location("reference_test_vis_gpu", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.vis_cpu


def main(ref_root):
    from hera_gpu_gb300 import synth

    vis_cpu = load_reference_vis_cpu(ref_root)
    out = {}

    # 1. the small configuration (16 ant x 1000 src x 10 times, 150 MHz)
    c = synth.config_small(seed=0)
    args = (c["antpos"], float(c["freqs"][0]), c["eq2tops"], c["crd_eq"],
            c["I_sky"], c["bm_cubes"][0])
    np.savez_compressed(
        os.path.join(HERE, "small_config.npz"),
        antpos=args[0], freq=args[1], eq2tops=args[2], crd_eq=args[3],
        I_sky=args[4], bm_cube=args[5],
        vis_p1=vis_cpu(*args, precision=1), vis_p2=vis_cpu(*args, precision=2))

    # 2. the reference's random comparison inputs (test_vis_gpu.py:245-276):
    #    rand() antpos / eq2tops / crd_eq / I_sky / beams, freq in [0, 1)
    rng = np.random.default_rng(1)
    nant, ntimes, P, npix = 16, 10, 31, 12 * 16 ** 2
    a = rng.random((nant, 3))
    e = rng.random((ntimes, 3, 3))
    s = rng.random((3, npix))
    i = rng.random(npix)
    b = rng.random((nant, P, P))
    f = float(rng.random())
    np.savez_compressed(
        os.path.join(HERE, "random_inputs.npz"), antpos=a, freq=f, eq2tops=e,
        crd_eq=s, I_sky=i, bm_cube=b,
        vis_p1=vis_cpu(a, f, e, s, i, b, precision=1),
        vis_p2=vis_cpu(a, f, e, s, i, b, precision=2))

    # 3. edges: sources on and past the beam grid edge (|l|,|m| >= 1 after a
    #    non-orthogonal eq2top), a 2-pixel beam, km-scale baselines at 200 MHz
    rng = np.random.default_rng(2)
    nant, ntimes, P, nsrc = 7, 3, 2, 257
    a = rng.normal(0, 800.0, (nant, 3))
    e = 1.3 * rng.normal(size=(ntimes, 3, 3))
    s = rng.normal(size=(3, nsrc))
    i = rng.random(nsrc) * 5
    b = rng.random((nant, P, P))
    f = 200e6
    np.savez_compressed(
        os.path.join(HERE, "edge_inputs.npz"), antpos=a, freq=f, eq2tops=e,
        crd_eq=s, I_sky=i, bm_cube=b,
        vis_p1=vis_cpu(a, f, e, s, i, b, precision=1),
        vis_p2=vis_cpu(a, f, e, s, i, b, precision=2))
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <root of the hera_gpu sources>")
    main(sys.argv[1])
