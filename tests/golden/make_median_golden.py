"""Generate the median-filter fixture in this folder from the reference itself.

Runs the reference's own ``MedianFilter`` (hera_gpu/median_filter.py:8-365:
its padding and stream loop, and its ``mf`` kernel with ``FloydWirth_kth``,
executed on the CPU by oracle/median_ref.py) on seeded images -- integer
valued, so that ties are common, and with negative values -- for odd, even
and one-dimensional windows, one image and a list of three, and stores
inputs and outputs in ``median_reference.npz``.  Even windows are the case
the reference's own tests cannot check (scipy's medfilt2d refuses them).

Usage (needs the reference sources; the fixture is committed, so the GPU
machine never runs this):

    python tests/golden/make_median_golden.py /path/to/reference
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.median_ref import reference_median_filter  # noqa: E402

WINDOWS = [(3, 3), (5, 5), (4, 2), (2, 4), (2, 2), (6, 6), (1, 4), (4, 1), (3, 7), (9, 5),
           (1, 1)]


def main(ref_root):
    rng = np.random.default_rng(2024)
    out = {}
    for n, (k0, k1) in enumerate(WINDOWS):
        shape = (int(rng.integers(1, 40)), int(rng.integers(1, 60))) if n % 3 == 2 else (29, 41)
        nimg = 3 if n % 2 else 1
        imgs = np.round(rng.normal(0, 3, (nimg,) + shape)).astype(np.float32)
        res = reference_median_filter(ref_root, input=imgs if nimg > 1 else imgs[0],
                                      kernel_size=[k0, k1])
        out[f"in_{n}"] = imgs
        out[f"window_{n}"] = np.array([k0, k1])
        out[f"out_{n}"] = np.stack(res)
        print((k0, k1), imgs.shape)
    np.savez_compressed(os.path.join(HERE, "median_reference.npz"), **out)


if __name__ == "__main__":
    main(sys.argv[1])
