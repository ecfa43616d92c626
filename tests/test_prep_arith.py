"""The FP32 arithmetic of the source preparation, restated on the CPU.

For FP32 inputs the preparation kernels (hera_gpu_gb300/csrc/hv_prep.cu:
dot3, above_horizon, beam_axis) form each topocentric component as an
unevaluated sum hi + lo with error-free transformations (TwoProduct by FMA,
TwoSum: the compensated dot product Dot2 of Ogita, Rump and Oishi, 2005), and
carry the beam coordinate (P - 1)(c / 2 + 1 / 2) as a float-float sum until
the weight is rounded once.  This test restates those steps in numpy with
every operation rounded to float32 (products exact in float64, the FMA's sum
in long double), and checks them against the FP64 evaluation the kernels used
before: the same horizon decisions, the same beam pixels, and weights within
half an FP32 unit of a long-double evaluation.
"""
import numpy as np
import pytest

f32 = np.float32


def _add(a, b):
    return (a.astype(np.float32) + b.astype(np.float32)).astype(np.float32)


def _sub(a, b):
    return (a.astype(np.float32) - b.astype(np.float32)).astype(np.float32)


def two_prod(a, b):
    p = (a * b).astype(np.float32)
    return p, (a.astype(np.float64) * b.astype(np.float64) - p.astype(np.float64)).astype(np.float32)


def two_sum(a, b):
    s = _add(a, b)
    bv = _sub(s, a)
    return s, _add(_sub(a, _sub(s, bv)), _sub(b, bv))


def fma32(a, b, c):
    L = np.longdouble
    return (L(1) * a.astype(L) * b.astype(L) + c.astype(L)).astype(np.float32)


def dot3(r, x, y, z):
    p, s = two_prod(np.full_like(x, r[0]), x)
    h, e = two_prod(np.full_like(y, r[1]), y)
    p, q = two_sum(p, h)
    s = _add(s, _add(q, e))
    h, e = two_prod(np.full_like(z, r[2]), z)
    p, q = two_sum(p, h)
    s = _add(s, _add(q, e))
    return two_sum(p, s)


def beam_axis_ff(hi, lo, P):
    h = np.full_like(hi, f32(0.5) * f32(P - 1))
    u, ue = two_sum(hi, np.ones_like(hi))
    ue = _add(ue, lo)
    b, be = two_prod(h, u)
    be = fma32(h, ue, be)
    fb = np.floor(b).astype(np.float32)
    f = _add(_sub(b, fb), be)
    low, high = f < 0, f >= 1
    fb = np.where(low, fb - 1, np.where(high, fb + 1, fb))
    f = np.where(low, _add(f, np.ones_like(f)), np.where(high, _sub(f, np.ones_like(f)), f))
    w = np.where(fb < 0, f32(0), np.where(fb >= P - 1, f32(1), f)).astype(np.float32)
    return np.clip(fb, 0, P - 2).astype(int), w


def beam_axis_f64(c, P):
    b = (P - 1) * (0.5 * c + 0.5)
    fb = np.floor(b)
    w = np.where(fb < 0, 0.0, np.where(fb >= P - 1, 1.0, b - fb))
    return np.clip(fb, 0, P - 2).astype(int), w


@pytest.mark.parametrize("P", [2, 31, 63, 1024])
def test_fp32_geometry_matches_fp64(P):
    rng = np.random.default_rng(P)
    n = 50_000
    for _ in range(2):
        Q = np.linalg.qr(rng.normal(size=(3, 3)))[0].astype(np.float32)
        v = rng.normal(size=(3, n))
        x, y, z = (v / np.linalg.norm(v, axis=0)).astype(np.float32)
        t64 = [Q[i, 0].astype(np.float64) * x + (Q[i, 1].astype(np.float64) * y
                                                  + Q[i, 2].astype(np.float64) * z)
               for i in range(3)]
        hz, _ = dot3(Q[2], x, y, z)
        np.testing.assert_array_equal(hz > 0, t64[2] > 0)          # horizon
        L = np.longdouble
        for ax in (0, 1):
            hi, lo = dot3(Q[ax], x, y, z)
            i32, w32 = beam_axis_ff(hi, lo, P)
            i64, w64 = beam_axis_f64(t64[ax], P)
            # the same texel, or the same point as (corner - 1, weight 1)
            same = ((i32 == i64) | ((i32 == i64 - 1) & (w32 == 1) & (w64 == 0))
                    | ((i64 == i32 - 1) & (w64 == 1) & (w32 == 0)))
            assert same.all()
            c = (Q[ax, 0].astype(L) * x.astype(L) + Q[ax, 1].astype(L) * y.astype(L)
                 + Q[ax, 2].astype(L) * z.astype(L))
            b = (L(P - 1) / 2) * (c + 1)
            inside = (np.floor(b) == i32) & (np.floor(b) >= 0) & (np.floor(b) <= P - 2)
            err = np.abs(w32[inside].astype(L) - (b - np.floor(b))[inside])
            assert float(err.max()) <= 2.0 ** -24 * 1.25


def _block_sort(keys, n, threads=1024):
    """hv_prep.cu:block_sort restated: thread i < n keeps the minimum of the
    pair (i, i ^ j) when its lower index sorts ascending ((i & k) == 0)."""
    w = np.full(threads, 0xffffffff, dtype=np.uint64)
    w[:len(keys)] = keys
    i = np.arange(threads)
    act = i < n
    k = 2
    while k <= n:
        j = k >> 1
        while j > 0:
            o = np.where(act, w[np.where(act, i ^ j, i)], w)
            keep_min = ((i & j) == 0) == ((i & k) == 0)
            w = np.where(act, np.where(keep_min, np.minimum(w, o), np.maximum(w, o)), w)
            j >>= 1
        k <<= 1
    return w


@pytest.mark.parametrize("total", [0, 1, 7, 31, 32, 33, 100, 511, 512, 700, 1024])
def test_pixel_order_sort_of_a_block(total):
    """The records of a preparation block in beam-pixel order, ties in
    catalogue order: keys (pixel << 10 | rank), a network of the smallest
    power of two >= max(total, 32) keys."""
    rng = np.random.default_rng(total)
    pix = rng.integers(0, 9, total).astype(np.uint64) + np.uint64(4000)
    keys = (pix << np.uint64(10)) | np.arange(total, dtype=np.uint64)
    n = 32
    while n < total:
        n <<= 1
    out = _block_sort(keys, n)[:total]
    np.testing.assert_array_equal(out, np.sort(keys))
    order = (out & np.uint64(1023)).astype(int)
    # stable: within a pixel, catalogue (rank) order
    np.testing.assert_array_equal(order, np.lexsort((np.arange(total), pix)))
