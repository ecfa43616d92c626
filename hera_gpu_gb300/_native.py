"""ctypes binding of libheravis.so (the C ABI declared in include/heravis.h).

The library is the only compute path: if it is missing, or no CUDA device is
usable, every call raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading
import weakref

import numpy as np

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libheravis.so")

HV_OK = 0
HV_ERR_ARG = 1
HV_ERR_OOM = 2
HV_ERR_CUDA = 3
HV_ERR_TIMEOUT = 4
HV_ERR_UNSUPPORTED = 5

METHODS = {"auto": 0, "plain": 1, "tc": 2, "tc_bf16": 2, "tc_fp16": 3}

class HvSim(ctypes.Structure):
    """hv_sim of include/heravis.h: one simulation of a batch (device
    pointers, except freqs which is a host pointer)."""
    _fields_ = [("antpos", ctypes.c_void_p), ("eq2tops", ctypes.c_void_p),
                ("crd_eq", ctypes.c_void_p), ("I_sky", ctypes.c_void_p),
                ("bm_cubes", ctypes.c_void_p), ("freqs", ctypes.c_void_p),
                ("vis_out", ctypes.c_void_p), ("nant", ctypes.c_int), ("ntimes", ctypes.c_int),
                ("nsrc", ctypes.c_int), ("nfreq", ctypes.c_int), ("beam_px", ctypes.c_int)]


HV_BATCH_GRAPH = 1
HV_BATCH_AUTOTUNE = 2

HV_TUNE_STAGES = 2

# Every function of the ABI: name -> (restype, argtypes)
_c_int, _c_void_p, _c_size_t, _c_double = ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_double
_PTR = ctypes.c_void_p
SIGNATURES = {
    "hv_version": (_c_int, []),
    "hv_create": (_c_int, [ctypes.POINTER(_c_void_p), _c_int, _c_size_t]),
    "hv_destroy": (_c_int, [_c_void_p]),
    "hv_last_error": (ctypes.c_char_p, [_c_void_p]),
    "hv_launch_count": (ctypes.c_uint64, [_c_void_p]),
    "hv_vis_gpu": (_c_int, [_c_void_p, _c_int, _c_int, _PTR, _c_int, _c_double, _PTR, _c_int,
                            _PTR, _PTR, _c_int, _PTR, _c_int, _PTR]),
    "hv_vis_multifreq": (_c_int, [_c_void_p, _c_int, _c_int, _PTR, _c_int, _PTR, _c_int, _PTR,
                                  _c_int, _PTR, _PTR, _c_int, _PTR, _c_int, _PTR]),
    "hv_vis_multifreq_device": (_c_int, [_c_void_p, _c_int, _c_int, _PTR, _c_int, _PTR, _c_int,
                                         _PTR, _c_int, _PTR, _PTR, _c_int, _PTR, _c_int, _PTR,
                                         _c_void_p]),
    "hv_sync": (_c_int, [_c_void_p]),
    "hv_set_profiling": (_c_int, [_c_void_p, _c_int]),
    "hv_profile_read": (_c_int, [_c_void_p, ctypes.POINTER(_c_double), ctypes.POINTER(ctypes.c_uint64)]),
    "hv_set_wait_limit": (_c_int, [_c_void_p, ctypes.c_uint64, _c_int]),
    "hv_set_tuning": (_c_int, [_c_void_p, _c_int, _c_int]),
    "hv_median_filter": (_c_int, [_c_void_p, _PTR, _PTR, _c_int, _c_int, _c_int, _c_int, _c_int]),
    "hv_median_filter_device": (_c_int, [_c_void_p, _PTR, _PTR, _c_int, _c_int, _c_int, _c_int,
                                         _c_int, _c_void_p]),
    "hv_omnical": (_c_int, [_c_void_p, _c_int, _PTR, _c_int, _PTR, _c_int, _PTR, _c_int, _PTR,
                            _PTR, _c_int, _c_double, _c_int, _c_int, _c_int, _c_double, _PTR,
                            _PTR, _PTR]),
    "hv_omnical_device": (_c_int, [_c_void_p, _c_int, _PTR, _c_int, _PTR, _c_int, _PTR, _c_int,
                                   _PTR, _PTR, _c_int, _c_double, _c_int, _c_int, _c_int,
                                   _c_double, _PTR, _PTR, _PTR, _c_void_p]),
    "hv_vis_gpu_noalloc": (_c_int, [_PTR, _c_int, _c_double, _PTR, _c_int, _PTR, _PTR, _c_int,
                                    _PTR, _c_int, _PTR, _c_void_p, ctypes.c_char_p, _c_size_t]),
    "hv_batch_create": (_c_int, [_c_void_p, ctypes.POINTER(HvSim), _c_int, ctypes.c_uint,
                                 ctypes.POINTER(_c_void_p)]),
    "hv_batch_launch": (_c_int, [_c_void_p, _c_void_p]),
    "hv_batch_sync": (_c_int, [_c_void_p]),
    "hv_batch_launches": (ctypes.c_uint64, [_c_void_p]),
    "hv_batch_destroy": (_c_int, [_c_void_p]),
    "hv_vis_batch": (_c_int, [_c_void_p, ctypes.POINTER(HvSim), _c_int, _c_void_p]),
    "hv_device_alloc": (_c_int, [_c_void_p, _c_size_t, ctypes.POINTER(_c_void_p)]),
    "hv_device_free": (_c_int, [_c_void_p, _c_void_p]),
    "hv_memcpy_async": (_c_int, [_c_void_p, _c_void_p, _c_void_p, _c_size_t, _c_int]),
    "hv_stream_query": (_c_int, [_c_void_p]),
    "hv_host_alloc": (_c_int, [_c_void_p, _c_size_t, ctypes.POINTER(_c_void_p)]),
    "hv_host_free": (_c_int, [_c_void_p, _c_void_p]),
}


class HeraVisError(RuntimeError):
    """A failed library call; ``code`` is the hv_status."""

    def __init__(self, code, msg):
        super().__init__(f"[hv_status {code}] {msg}")
        self.code = code


class HeraVisArgumentError(HeraVisError, AssertionError):
    """Bad shape or argument (the reference raises AssertionError here)."""


class HeraVisTimeout(HeraVisError):
    """A bounded device-side wait gave up; the GPU context stays usable."""


_lib = None
_lib_lock = threading.Lock()


def load_library(path: str = LIB_PATH):
    """Load libheravis.so and declare its ABI.  Raises if it is missing."""
    global _lib
    with _lib_lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise RuntimeError(
                f"libheravis.so not found at {path}: build it with "
                "`python -m hera_gpu_gb300.build` (nvcc, sm_103a). There is no CPU fallback.")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else ctypes.c_void_p(0)


class Context:
    """One hv_context: a CUDA device, a stream and a workspace."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        rc = self.lib.hv_create(ctypes.byref(h), int(device), int(hbm_budget_bytes))
        if rc != HV_OK:
            if rc == HV_ERR_UNSUPPORTED:
                raise HeraVisError(rc, "no CUDA device available: libheravis needs a GB300 GPU")
            raise HeraVisError(rc, f"hv_create(device={device}) failed")
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self.lib.hv_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc):
        if rc == HV_OK:
            return
        msg = self.lib.hv_last_error(self.h).decode(errors="replace")
        if rc == HV_ERR_ARG:
            raise HeraVisArgumentError(rc, msg)
        if rc == HV_ERR_TIMEOUT:
            raise HeraVisTimeout(rc, msg)
        raise HeraVisError(rc, msg)

    @property
    def launches(self) -> int:
        return int(self.lib.hv_launch_count(self.h))

    def sync(self):
        self.check(self.lib.hv_sync(self.h))

    def vis_multifreq(self, precision, method, antpos, freqs, eq2tops, crd_eq, I_sky, bm_cubes, out):
        """Host arrays in, host array ``out`` (nfreq, ntimes, nant, nant) written."""
        freqs = np.ascontiguousarray(freqs, dtype=np.float64)
        nant = antpos.shape[0]
        rc = self.lib.hv_vis_multifreq(
            self.h, int(precision), METHODS[method], _ptr(antpos), nant, _ptr(freqs), len(freqs),
            _ptr(eq2tops), eq2tops.shape[0], _ptr(crd_eq), _ptr(I_sky), crd_eq.shape[1],
            _ptr(bm_cubes), bm_cubes.shape[-1], _ptr(out))
        self.check(rc)
        return out

    def vis_multifreq_device(self, precision, method, d_antpos, nant, freqs, d_eq2tops, ntimes,
                             d_crd_eq, d_I_sky, nsrc, d_bm_cubes, beam_px, d_out, stream=0):
        """Device pointers (ints) in and out; asynchronous on ``stream``."""
        freqs = np.ascontiguousarray(freqs, dtype=np.float64)
        rc = self.lib.hv_vis_multifreq_device(
            self.h, int(precision), METHODS[method], ctypes.c_void_p(d_antpos), int(nant),
            _ptr(freqs), len(freqs), ctypes.c_void_p(d_eq2tops), int(ntimes),
            ctypes.c_void_p(d_crd_eq), ctypes.c_void_p(d_I_sky), int(nsrc),
            ctypes.c_void_p(d_bm_cubes), int(beam_px), ctypes.c_void_p(d_out),
            ctypes.c_void_p(stream))
        self.check(rc)

    def device_alloc(self, nbytes: int) -> int:
        p = ctypes.c_void_p()
        self.check(self.lib.hv_device_alloc(self.h, int(nbytes), ctypes.byref(p)))
        return int(p.value or 0)

    def device_free(self, ptr: int):
        self.check(self.lib.hv_device_free(self.h, ctypes.c_void_p(ptr)))

    def h2d(self, dst: int, src: np.ndarray):
        """Asynchronous copy on the context's stream (src must stay alive
        until the stream has passed it; page-locked for true overlap)."""
        self.check(self.lib.hv_memcpy_async(self.h, ctypes.c_void_p(dst), _ptr(src), src.nbytes, 1))

    def d2h(self, dst: np.ndarray, src: int):
        self.check(self.lib.hv_memcpy_async(self.h, _ptr(dst), ctypes.c_void_p(src), dst.nbytes, 2))

    def idle(self) -> bool:
        """True once all work queued on the context's stream has finished."""
        r = self.lib.hv_stream_query(self.h)
        if r < 0:
            self.check(-r)
        return r == 0

    def set_profiling(self, enable: bool):
        self.check(self.lib.hv_set_profiling(self.h, 1 if enable else 0))

    def set_wait_limit(self, wait_s: float = 0.0, stall: bool = False):
        """Limit of each device-side wait of the fused kernel (0: 10 s); with
        ``stall`` the next fused launches are made to time out (fault
        injection for tests of failure detection)."""
        self.check(self.lib.hv_set_wait_limit(self.h, int(wait_s * 1e9), 1 if stall else 0))

    def set_tuning(self, stages: int = 0):
        """Launch shape of the fused kernel for later calls (hv_set_tuning;
        0 = the default)."""
        self.check(self.lib.hv_set_tuning(self.h, HV_TUNE_STAGES, int(stages)))

    def median_filter(self, images, out, k0, k1):
        """Median filter of the (nimg, rows, cols) float32 images into out
        (hv_median_filter)."""
        assert images.dtype == np.float32 and out.dtype == np.float32
        assert images.flags.c_contiguous and out.flags.c_contiguous and images.shape == out.shape
        n, rows, cols = images.shape
        self.check(self.lib.hv_median_filter(self.h, _ptr(images), _ptr(out), n, rows, cols,
                                             int(k0), int(k1)))

    def omnical(self, precision, ggu, gains, ubls, data, wgts, conv_crit, maxiter, check_every,
                check_after, gain, chisq, iters, conv):
        """Omnical on host arrays (hv_omnical): gains and ubls are updated in
        place; chisq, iters and conv are filled."""
        rt, ct = (np.float32, np.complex64) if precision == 1 else (np.float64, np.complex128)
        for a, t in ((gains, ct), (ubls, ct), (data, ct), (wgts, rt), (chisq, rt), (conv, rt),
                     (iters, np.uint32), (ggu, np.uint32)):
            assert a.dtype == t and a.flags.c_contiguous
        ndata, nants = gains.shape
        self.check(self.lib.hv_omnical(self.h, int(precision), _ptr(ggu), ggu.shape[0],
                                       _ptr(gains), nants, _ptr(ubls), ubls.shape[1], _ptr(data),
                                       _ptr(wgts), ndata, float(conv_crit), int(maxiter),
                                       int(check_every), int(check_after), float(gain),
                                       _ptr(chisq), _ptr(iters), _ptr(conv)))

    def profile_read(self):
        """(milliseconds, launches) of the visibility-product kernels since
        the last read (CUDA events on their stream)."""
        ms = ctypes.c_double()
        n = ctypes.c_uint64()
        self.check(self.lib.hv_profile_read(self.h, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, int(n.value)

    def pinned_empty(self, shape, dtype):
        """A numpy array in page-locked host memory, freed when the last view
        of it is gone."""
        dtype = np.dtype(dtype)
        n = int(np.prod(shape))
        nbytes = max(n * dtype.itemsize, 1)
        p = ctypes.c_void_p()
        self.check(self.lib.hv_host_alloc(self.h, nbytes, ctypes.byref(p)))
        buf = (ctypes.c_byte * nbytes).from_address(p.value)
        weakref.finalize(buf, self.lib.hv_host_free, self.h, ctypes.c_void_p(p.value))
        return np.frombuffer(buf, dtype=dtype, count=n).reshape(shape)


class Batch:
    """A planned batch of simulations (hv_batch_create).  ``sims`` is a list
    of dicts of device pointers / sizes (see HvSim); ``freqs`` of each is a
    numpy float64 array kept alive here."""

    def __init__(self, ctx: "Context", sims, graph=False, autotune=False):
        self.ctx = ctx
        self._freqs = [np.ascontiguousarray(s["freqs"], dtype=np.float64) for s in sims]
        arr = (HvSim * len(sims))()
        for i, s in enumerate(sims):
            arr[i] = HvSim(s["antpos"], s["eq2tops"], s["crd_eq"], s["I_sky"], s["bm_cubes"],
                           self._freqs[i].ctypes.data, s["vis_out"], s["nant"], s["ntimes"],
                           s["nsrc"], len(self._freqs[i]), s["beam_px"])
        self._arr = arr
        h = ctypes.c_void_p()
        flags = (HV_BATCH_GRAPH if graph else 0) | (HV_BATCH_AUTOTUNE if autotune else 0)
        ctx.check(ctx.lib.hv_batch_create(ctx.h, arr, len(sims), flags, ctypes.byref(h)))
        self.h = h

    @property
    def launches(self) -> int:
        return int(self.ctx.lib.hv_batch_launches(self.h))

    def launch(self, stream=0):
        self.ctx.check(self.ctx.lib.hv_batch_launch(self.h, ctypes.c_void_p(stream)))

    def sync(self):
        self.ctx.check(self.ctx.lib.hv_batch_sync(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.hv_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_contexts = {}
_ctx_lock = threading.Lock()


def default_context(device: int = 0) -> Context:
    """Process-wide context per device, created on first use (the reference
    binds device 0 at import through pycuda.autoinit, vis.py:1)."""
    with _ctx_lock:
        ctx = _contexts.get(device)
        if ctx is None:
            ctx = Context(device)
            _contexts[device] = ctx
        return ctx
