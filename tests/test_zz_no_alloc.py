"""The allocation-free entry point hv_vis_gpu_noalloc, through the C ABI.

Callers that cannot allocate device memory at call time (a pipeline whose
device memory is fixed up front, a framework that owns the allocator) use
this entry point; its working memory is a fixed array inside the library.
It runs the same kernels in the same order as the allocating plain form, so
its output must equal that form's bit for bit, on every call (the array
keeps the previous call's contents), and agree with the FP64 oracle within
the plain FP32 tolerance.  A request whose working memory is just under the
array's size checks the layout of the regions up to the array's end.  This
file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from noalloc_sizes import SCRATCH_BYTES, largest_nsrc, need_bytes

pytestmark = pytest.mark.gpu

TOL = 1e-5  # the plain FP32 tolerance of the parity tests
FREQ = 150e6


def _inputs(seed, nant, nsrc, ntimes, P):
    from hera_gpu_gb300 import synth
    rng = np.random.default_rng(seed)
    antpos = rng.normal(0, 80.0, (nant, 3)).astype(np.float32)
    crd = synth.sphere_sources(nsrc, rng).astype(np.float32)
    I = (rng.random(nsrc) * 3).astype(np.float32)
    bm = rng.random((nant, P, P)).astype(np.float32)
    e2t = np.stack([np.linalg.qr(rng.normal(size=(3, 3)))[0] for _ in range(ntimes)]).astype(np.float32)
    return antpos, e2t, crd, I, bm


def _both(ctx, lib, stream, dev, case):
    """(no-alloc output, allocating plain output, inputs) of one request."""
    import torch
    seed, nant, nsrc, ntimes, P = case
    host = _inputs(seed, nant, nsrc, ntimes, P)
    antpos, e2t, crd, I, bm = host
    d = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in host]
    ref = torch.empty((1, ntimes, nant, nant), dtype=torch.complex64, device=dev)
    torch.cuda.synchronize()
    ctx.vis_multifreq_device(1, "plain", d[0].data_ptr(), nant, [FREQ], d[1].data_ptr(),
                             ntimes, d[2].data_ptr(), d[3].data_ptr(), nsrc, d[4].data_ptr(),
                             P, ref.data_ptr(), stream.cuda_stream)
    ctx.sync()
    torch.cuda.synchronize()
    out = torch.full((ntimes, nant, nant), float("nan"), dtype=torch.complex64, device=dev)
    err = ctypes.create_string_buffer(512)
    rc = lib.hv_vis_gpu_noalloc(
        ctypes.c_void_p(d[0].data_ptr()), nant, FREQ, ctypes.c_void_p(d[1].data_ptr()),
        ntimes, ctypes.c_void_p(d[2].data_ptr()), ctypes.c_void_p(d[3].data_ptr()), nsrc,
        ctypes.c_void_p(d[4].data_ptr()), P, ctypes.c_void_p(out.data_ptr()),
        ctypes.c_void_p(stream.cuda_stream), err, len(err))
    assert rc == 0, err.value.decode()
    stream.synchronize()
    return out.cpu().numpy(), ref[0].cpu().numpy(), host


def _check(case, a, b, host):
    from oracle import rel_frobenius, vis_oracle
    assert np.all(np.isfinite(a)), f"{case}: unwritten output"
    np.testing.assert_array_equal(a, b, err_msg=f"{case}: differs from the plain form")
    antpos, e2t, crd, I, bm = (x.astype(np.float64) for x in host)
    ref = vis_oracle(antpos, FREQ, e2t, crd, I, bm)
    err = rel_frobenius(a, ref).max()
    assert err <= TOL, f"{case}: {err:.2e} vs the FP64 oracle"


def test_no_alloc_matches_allocating_entry_point_twice():
    import torch
    from hera_gpu_gb300 import _native
    lib = _native.load_library()
    ctx = _native.Context(0)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    for case in [(1, 40, 3000, 3, 31), (2, 150, 5000, 2, 15)]:
        a, b, host = _both(ctx, lib, stream, dev, case)
        _check(case, a, b, host)


def test_no_alloc_at_the_size_limit():
    import torch
    from hera_gpu_gb300 import _native
    lib = _native.load_library()
    ctx = _native.Context(0)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    nant, ntimes, P = 150, 2, 31
    nsrc = largest_nsrc(nant, ntimes, P)
    need = need_bytes(nant, nsrc, ntimes, P)
    assert SCRATCH_BYTES - 65536 < need <= SCRATCH_BYTES
    case = (5, nant, nsrc, ntimes, P)
    a, b, host = _both(ctx, lib, stream, dev, case)
    _check(case, a, b, host)


def test_no_alloc_rejects_oversize_requests():
    from hera_gpu_gb300 import _native
    lib = _native.load_library()
    err = ctypes.create_string_buffer(512)
    one = ctypes.c_void_p(1)  # never dereferenced: the size check comes first
    rc = lib.hv_vis_gpu_noalloc(one, 350, 150e6, one, 1, one, one, 1_000_000, one, 63, one,
                                ctypes.c_void_p(0), err, len(err))
    assert rc == _native.HV_ERR_ARG
    assert b"working memory" in err.value
