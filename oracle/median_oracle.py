"""CPU oracle of hera_gpu's 2-D median filter -- TEST INFRASTRUCTURE ONLY.

Restates hera_gpu/median_filter.py:8-365 in numpy: every image is padded by
zeros, k0 // 2 rows above and below and k1 // 2 columns left and right
(median_filter.py:23-25, 318); the window of output pixel (r, c) covers padded
rows r .. r + k0 - 1 and columns c .. c + k1 - 1 (median_filter.py:223-230,
the loops of `mf` over fx, fy offset by the half windows); the output is the
window's element of rank floor(k0 * k1 / 2) in ascending order
(median_filter.py:252, FloydWirth_kth(window, WS^2 / 2)), computed in float32
(median_filter.py:318).  The result is cropped back to the image's shape
(median_filter.py:360-363).

Pinned by the reference's own test oracle (hera_gpu/tests/test_median_filter.py
compares with scipy.signal.medfilt2d), which agrees with this restatement for
odd windows, and by the reference's own MedianFilter run on the CPU
(oracle/median_ref.py; tests/golden/median_reference.npz), bit for bit for
odd, even and one-dimensional windows; tests/test_median.py checks both.
Only tests/ and bench.py's CPU baseline use this module.
"""
import numpy as np


def median_filter_oracle(image, k0, k1):
    """The rank-floor(k0 * k1 / 2) element of each zero-padded k0 x k1 window."""
    a = np.asarray(image, dtype=np.float32)
    rows, cols = a.shape
    p0, p1 = k0 // 2, k1 // 2
    # pad so that every window lies inside (k0 - 1 - p0 below, k1 - 1 - p1 right)
    pad = np.zeros((rows + k0 - 1, cols + k1 - 1), dtype=np.float32)
    pad[p0:p0 + rows, p1:p1 + cols] = a
    win = np.lib.stride_tricks.sliding_window_view(pad, (k0, k1))  # (rows, cols, k0, k1)
    flat = win.reshape(rows, cols, k0 * k1)
    k = (k0 * k1) // 2
    return np.partition(flat, k, axis=-1)[..., k]
