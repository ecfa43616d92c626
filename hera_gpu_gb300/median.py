"""Drop-in for hera_gpu's 2-D median filter (``hera_gpu.MedianFilter``).

The reference (hera_gpu/median_filter.py:8-365) takes one image or a list of
images of one shape, pads each with zeros by half the window
(median_filter.py:318), and returns a list of images whose pixels are the
element of rank floor(k0 * k1 / 2) of the k0 x k1 window centred on them;
for odd windows that is ``scipy.signal.medfilt2d``.  Here every image of the
call goes through one launch of libheravis.so's median kernel
(``hv_median_filter``).
"""
from __future__ import annotations

import numpy as np

from . import _native


def MedianFilter(input=None, kernel_size=3, bw=32, bh=32, context=None):
    """Median filter of ``input`` (an image, a list of images of one shape, or
    an (nimg, rows, cols) array) with a ``kernel_size`` window (an int, or
    (rows, columns)).  Returns a list of float32 images, as the reference
    (a single image comes back as a list of one).  ``bw``/``bh`` (the
    reference's block shape) are accepted and not needed."""
    if isinstance(kernel_size, (int, np.integer)):
        kernel_size = [int(kernel_size)] * 2
    k0, k1 = (int(k) for k in kernel_size)
    assert k0 >= 1 and k1 >= 1, "window sizes must be positive"
    images = np.asarray(input)
    assert images.ndim in (2, 3), "expects an image or a list of images of one shape"
    if images.ndim == 2:
        images = images[None]
    images = np.ascontiguousarray(images, dtype=np.float32)
    out = np.empty_like(images)
    ctx = context or _native.default_context()
    ctx.median_filter(images, out, k0, k1)
    return [out[i] for i in range(out.shape[0])]
