"""The reference's own MedianFilter, run on the CPU -- TEST INFRASTRUCTURE
ONLY.

Runs the unmodified ``MedianFilter`` of hera_gpu/median_filter.py:8-365 --
its padding, launch geometry and stream loop, and its ``mf`` kernel with
``FloydWirth_kth`` (median_filter.py:96-216) -- without a GPU, to produce
reference outputs for tests/golden/ (make_median_golden.py).  The pycuda
calls it makes are stubbed: device allocations and page-locked buffers are
numpy arrays, copies are memory copies, streams do nothing, and
``SourceModule`` is oracle/cuda_emu.py (the kernel source as the reference
formats it, compiled with g++ for the host; a launch runs every thread in
turn).  Needs the reference sources; the tests use the fixtures it made.
"""
from __future__ import annotations

import contextlib
import importlib.util
import os
import sys
import types

import numpy as np

from . import cuda_emu


class _DeviceBuffer:
    def __init__(self, nbytes):
        self.arr = np.zeros(nbytes, dtype=np.uint8)


def _htod(dst, src, stream=None):
    dst.arr[:] = np.ascontiguousarray(src).view(np.uint8).reshape(-1)


def _dtoh(dst, src, stream=None):
    dst.view(np.uint8).reshape(-1)[:] = src.arr


@contextlib.contextmanager
def _stubs():
    mods = {}
    pycuda = types.ModuleType("pycuda")
    mods["pycuda"] = pycuda
    for sub in ("autoinit", "compiler", "driver"):
        m = types.ModuleType("pycuda." + sub)
        setattr(pycuda, sub, m)
        mods["pycuda." + sub] = m
    mods["pycuda.compiler"].SourceModule = lambda code: cuda_emu.Module(code)
    drv = mods["pycuda.driver"]
    drv.Stream = lambda: None
    drv.register_host_memory = lambda a: a
    drv.pagelocked_empty_like = np.empty_like
    drv.mem_alloc = _DeviceBuffer
    drv.memcpy_htod_async = _htod
    drv.memcpy_dtoh_async = _dtoh
    clash = [k for k in mods if k in sys.modules]
    assert not clash, f"real modules present: {clash}"
    sys.modules.update(mods)
    try:
        yield
    finally:
        for k in mods:
            sys.modules.pop(k, None)


def reference_median_filter(ref_root, *args, **kwargs):
    """hera_gpu.MedianFilter(*args, **kwargs) of the reference sources under
    ref_root, the reference's own code, on the CPU (see the module
    docstring)."""
    with _stubs():
        path = os.path.join(ref_root, "hera_gpu", "median_filter.py")
        spec = importlib.util.spec_from_file_location("_reference_median_filter", path)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        return mod.MedianFilter(*args, **kwargs)
