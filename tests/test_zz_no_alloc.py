"""The allocation-free entry point hv_vis_gpu_noalloc, through the C ABI.

Callers that cannot allocate device memory at call time (a pipeline whose
device memory is fixed up front, a framework that owns the allocator) use
this entry point; its working memory is a fixed array inside the library.
It must give what the allocating entry point gives for the same inputs, on
every call (the array keeps the previous call's contents), and refuse
requests larger than its array.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5  # the plain FP32 tolerance of the parity tests


def _inputs(seed, nant, nsrc, ntimes, P):
    from hera_gpu_gb300 import synth
    rng = np.random.default_rng(seed)
    antpos = rng.normal(0, 80.0, (nant, 3)).astype(np.float32)
    crd = synth.sphere_sources(nsrc, rng).astype(np.float32)
    I = (rng.random(nsrc) * 3).astype(np.float32)
    bm = rng.random((nant, P, P)).astype(np.float32)
    e2t = np.stack([np.linalg.qr(rng.normal(size=(3, 3)))[0] for _ in range(ntimes)]).astype(np.float32)
    return antpos, e2t, crd, I, bm


def test_no_alloc_matches_allocating_entry_point_twice():
    import torch
    from hera_gpu_gb300 import _native
    from oracle import rel_frobenius

    lib = _native.load_library()
    ctx = _native.Context(0)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    freq = 150e6
    for call, (seed, nant, nsrc, ntimes, P) in enumerate([(1, 40, 3000, 3, 31),
                                                           (2, 150, 5000, 2, 15)]):
        antpos, e2t, crd, I, bm = _inputs(seed, nant, nsrc, ntimes, P)
        d = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in (antpos, e2t, crd, I, bm)]
        ref = torch.empty((1, ntimes, nant, nant), dtype=torch.complex64, device=dev)
        torch.cuda.synchronize()
        ctx.vis_multifreq_device(1, "plain", d[0].data_ptr(), nant, [freq], d[1].data_ptr(),
                                 ntimes, d[2].data_ptr(), d[3].data_ptr(), nsrc, d[4].data_ptr(),
                                 P, ref.data_ptr(), stream.cuda_stream)
        ctx.sync()
        torch.cuda.synchronize()
        out = torch.full((ntimes, nant, nant), float("nan"), dtype=torch.complex64, device=dev)
        err = ctypes.create_string_buffer(512)
        rc = lib.hv_vis_gpu_noalloc(
            ctypes.c_void_p(d[0].data_ptr()), nant, freq, ctypes.c_void_p(d[1].data_ptr()),
            ntimes, ctypes.c_void_p(d[2].data_ptr()), ctypes.c_void_p(d[3].data_ptr()), nsrc,
            ctypes.c_void_p(d[4].data_ptr()), P, ctypes.c_void_p(out.data_ptr()),
            ctypes.c_void_p(stream.cuda_stream), err, len(err))
        assert rc == 0, err.value.decode()
        stream.synchronize()
        a = out.cpu().numpy()
        b = ref[0].cpu().numpy()
        assert np.all(np.isfinite(a)), f"call {call}: unwritten output"
        assert rel_frobenius(a, b).max() <= TOL, f"call {call}"


def test_no_alloc_rejects_oversize_requests():
    from hera_gpu_gb300 import _native
    lib = _native.load_library()
    err = ctypes.create_string_buffer(512)
    one = ctypes.c_void_p(1)  # never dereferenced: the size check comes first
    rc = lib.hv_vis_gpu_noalloc(one, 350, 150e6, one, 1, one, one, 1_000_000, one, 63, one,
                                ctypes.c_void_p(0), err, len(err))
    assert rc == _native.HV_ERR_ARG
    assert b"working memory" in err.value
