"""The 2-D median filter (hera_gpu.MedianFilter, median_filter.py:8-365).

CPU: the oracle restatement against scipy.signal.medfilt2d, the reference's
own test oracle (hera_gpu/tests/test_median_filter.py), including 1x1
images and windows larger than the image, and against the reference's own
MedianFilter run on the CPU (tests/golden/median_reference.npz, made by
make_median_golden.py), which also covers even windows.  GPU: the library's kernel against
the oracle, bit for bit (a median is a selection, no arithmetic), on the
reference's test shapes and windows, through the drop-in MedianFilter.
"""
import os
import zlib

import numpy as np
import pytest
import scipy.signal as sps

from oracle import median_filter_oracle

GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "median_reference.npz"))
REF_CASES = sorted(int(k[3:]) for k in GOLDEN.files if k.startswith("in_"))


@pytest.mark.parametrize("n", REF_CASES)
def test_oracle_matches_the_reference_median_filter(n):
    # the reference's own MedianFilter (its mf kernel, run on the CPU) on odd,
    # even and one-dimensional windows: equal bit for bit
    k0, k1 = (int(x) for x in GOLDEN[f"window_{n}"])
    for img, ref in zip(GOLDEN[f"in_{n}"], GOLDEN[f"out_{n}"]):
        np.testing.assert_array_equal(median_filter_oracle(img, k0, k1), ref)


ODD_CASES = [((1, 1), 1), ((29, 29), 1), ((29, 29), 3), ((93, 93), 3), ((1, 1), 3),
             ((1, 1), 9), ((40, 37), 5), ((1, 73), (1, 11)), ((5, 3), (11, 1)),
             ((2, 3), (3, 5)), ((60, 45), (9, 5)), ((31, 17), 9)]


@pytest.mark.parametrize("shape,ks", ODD_CASES)
def test_oracle_matches_scipy_medfilt2d(shape, ks):
    rng = np.random.default_rng(zlib.crc32(repr((shape, ks)).encode()))
    img = rng.random(shape).astype(np.float32)
    k0, k1 = (ks, ks) if isinstance(ks, int) else ks
    ref = sps.medfilt2d(img, (k0, k1))
    np.testing.assert_array_equal(median_filter_oracle(img, k0, k1), ref)


def test_oracle_even_window_follows_the_reference_rank():
    # an even window (scipy refuses it) takes the rank-(k0*k1)//2 element of
    # the window starting k//2 above/left, as the reference's kernel
    img = np.arange(16, dtype=np.float32).reshape(4, 4)
    out = median_filter_oracle(img, 2, 2)
    # pixel (1, 1): padded window rows 0..1 x cols 0..1 around it = {0, 1, 4, 5}
    assert out[1, 1] == 4.0


gpu = pytest.mark.gpu
REF_SHAPES = [((1, 1), 1), ((29, 29), 1), ((93, 93), 1), ((7000, 7000), 1),
              ((1, 1), 3), ((29, 29), 3), ((93, 93), 3), ((7000, 7000), 3),
              ((1, 1), 5), ((4000, 4000), 5), ((1, 1), 9), ((997, 997), 9),
              ((1, 73), 1), ((5, 3), 1), ((2, 3), 3), ((8013, 700), 5),
              ((1, 73), (1, 11)), ((5, 3), (11, 1)), ((2, 3), (3, 5)), ((8013, 700), (9, 5))]


@gpu
@pytest.mark.parametrize("shape,ks", REF_SHAPES)
def test_median_filter_matches_oracle(shape, ks):
    from hera_gpu_gb300 import MedianFilter
    rng = np.random.default_rng(7)
    img = rng.random(shape)
    k0, k1 = (ks, ks) if isinstance(ks, int) else ks
    out = MedianFilter(input=img, kernel_size=ks)
    assert isinstance(out, list) and len(out) == 1 and out[0].shape == shape
    ref = sps.medfilt2d(img.astype(np.float32), (k0, k1)) if max(shape) > 1000 else \
        median_filter_oracle(img, k0, k1)
    np.testing.assert_array_equal(out[0], ref)
    assert np.allclose(sps.medfilt2d(img, (k0, k1)), out)   # the reference's own check


@gpu
@pytest.mark.parametrize("n", REF_CASES)
def test_median_filter_matches_the_reference(n):
    # the library against the reference's own MedianFilter, bit for bit
    from hera_gpu_gb300 import MedianFilter
    k0, k1 = (int(x) for x in GOLDEN[f"window_{n}"])
    imgs = GOLDEN[f"in_{n}"]
    out = MedianFilter(input=imgs, kernel_size=(k0, k1))
    for got, ref in zip(out, GOLDEN[f"out_{n}"]):
        np.testing.assert_array_equal(got, ref)


@gpu
def test_median_filter_list_of_images_and_negative_values():
    from hera_gpu_gb300 import MedianFilter
    rng = np.random.default_rng(3)
    imgs = [rng.normal(0, 10, (50, 70)) for _ in range(5)]
    out = MedianFilter(input=imgs, kernel_size=(3, 7))
    assert len(out) == 5
    for a, b in zip(imgs, out):
        np.testing.assert_array_equal(b, median_filter_oracle(a, 3, 7))


@gpu
def test_median_filter_even_window_and_bad_window():
    from hera_gpu_gb300 import MedianFilter, _native
    img = np.random.default_rng(5).random((33, 21))
    np.testing.assert_array_equal(MedianFilter(input=img, kernel_size=(4, 2))[0],
                                  median_filter_oracle(img, 4, 2))
    with pytest.raises(_native.HeraVisError):
        MedianFilter(input=img, kernel_size=(301, 301))   # its tile exceeds shared memory


@gpu
@pytest.mark.parametrize("shape", [(16, 128), (17, 129), (31, 130), (33, 131), (2, 4), (300, 517),
                                   (32, 128), (65, 255)])
def test_median_3x3_kernel_edges(shape):
    # the 3 x 3 kernel's block edges (128 x 16 outputs), widths of every
    # residue mod 4 (float4 stores only when rows are 16-byte aligned),
    # several images in one launch, ties and negative values
    from hera_gpu_gb300 import MedianFilter
    rng = np.random.default_rng(shape[0] * 1000 + shape[1])
    imgs = np.round(rng.normal(0, 3, (3,) + shape)).astype(np.float32)
    out = MedianFilter(input=imgs, kernel_size=3)
    for a, b in zip(imgs, out):
        np.testing.assert_array_equal(b, median_filter_oracle(a, 3, 3))


@gpu
def test_median_3x3_unaligned_device_output():
    # hv_median_filter_device into an output that starts 4 bytes past a
    # 16-byte boundary: the kernel stores element by element
    import ctypes

    import torch
    from hera_gpu_gb300 import _native
    ctx = _native.default_context()
    img = np.random.default_rng(9).random((40, 64)).astype(np.float32)
    d_in = torch.from_numpy(img).cuda()
    d_out = torch.zeros(img.size + 1, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()  # the context's stream does not wait for torch's
    ctx.check(ctx.lib.hv_median_filter_device(
        ctx.h, ctypes.c_void_p(d_in.data_ptr()), ctypes.c_void_p(d_out.data_ptr() + 4), 1, 40, 64,
        3, 3, ctypes.c_void_p(0)))
    ctx.check(ctx.lib.hv_sync(ctx.h))
    got = d_out[1:].cpu().numpy().reshape(40, 64)
    np.testing.assert_array_equal(got, median_filter_oracle(img, 3, 3))
    assert float(d_out[0]) == 0.0


@gpu
@pytest.mark.parametrize("ks", [(5, 5), (7, 7), (9, 9), (9, 5), (5, 9)])
@pytest.mark.parametrize("shape", [(1, 1), (13, 11), (61, 47), (300, 129)])
def test_median_windows_forgetful(ks, shape):
    # the windows taken by forgetful selection: ties, negative values, zero
    # padding at every edge, several images a launch
    from hera_gpu_gb300 import MedianFilter
    rng = np.random.default_rng(ks[0] * 1000 + ks[1] * 100 + shape[0])
    imgs = np.round(rng.normal(0, 2, (2,) + shape)).astype(np.float32)
    out = MedianFilter(input=imgs, kernel_size=ks)
    for a, b in zip(imgs, out):
        np.testing.assert_array_equal(b, median_filter_oracle(a, *ks))
