"""The reference's own omnical, run on the CPU -- TEST INFRASTRUCTURE ONLY.

Runs the unmodified ``omnical`` of hera_gpu/redcal.py:358-743 (its host loop)
and its CUDA kernels (the GPU_TEMPLATE string, redcal.py:19-355) without a
GPU, to produce reference outputs for tests/golden/ (make_omnical_golden.py):

* the reference's imports are stubbed: pycuda arrays are numpy arrays
  (zero-filled, where pycuda's gpuarray.empty leaves memory as it finds it),
  events are no-ops, the two cuBLAS copies are memory copies, hera_cal's
  OmnicalSolver / RedundantCalibrator are empty base classes, and
  linsolve's get_name is its rule (a trailing '_' marks a conjugated
  variable and is not part of the name);
* ``SourceModule`` is oracle/cuda_emu.py: the kernel source exactly as the
  reference formats it, compiled with g++ for the host, a launch run as a
  loop over every thread -- blocks y-major, then threads y-major, so that in
  update_active (redcal.py:314-354) the thread with td == 0 of a pixel runs
  before the others that read the flag it writes, as the kernel's barrier
  orders them.

The atomic sums are thus taken in thread order, which the GPU does not fix;
their rounding differs from any one GPU run at the last bits.
``reference_solve_iteratively`` runs the reference's
``OmnicalSolverGPU.solve_iteratively`` (redcal.py:747-837) the same way, for
tests/golden/make_redcal_solver_golden.py.  Needs the reference sources; the
tests use the fixtures it made.
"""
from __future__ import annotations

import contextlib
import ctypes
import importlib.util
import os
import sys
import types

import numpy as np

from . import cuda_emu

# the template's atomicAdd(double) shim is for devices before sm_60
_DEFINES = "#define __CUDA_ARCH__ 800\n"


class _GPUArray:
    def __init__(self, shape, dtype):
        self.arr = np.zeros(shape, dtype=dtype)
        self.gpudata = self.arr.ctypes.data

    def set_async(self, a):
        self.arr[...] = a

    def get_async(self, ary=None):
        if ary is None:
            return self.arr.copy()
        np.copyto(ary, self.arr)
        return ary


class _Event:
    def record(self):
        pass

    def synchronize(self):
        pass

    def time_since(self, other):
        return 0.0


def _source_module(code):
    return cuda_emu.Module(code, includes="#include <cuComplex.h>", defines=_DEFINES)


def _copy(itemsize):
    def copy(handle, n, x, incx, y, incy):
        assert incx == 1 and incy == 1
        ctypes.memmove(y, x, n * itemsize)
    return copy


@contextlib.contextmanager
def _stubs():
    mods = {}
    pycuda = types.ModuleType("pycuda")
    mods["pycuda"] = pycuda
    for sub in ("autoinit", "compiler", "gpuarray", "driver"):
        m = types.ModuleType("pycuda." + sub)
        setattr(pycuda, sub, m)
        mods["pycuda." + sub] = m
    mods["pycuda.compiler"].SourceModule = _source_module
    mods["pycuda.gpuarray"].empty = lambda shape, dtype: _GPUArray(shape, dtype)
    mods["pycuda.driver"].Event = _Event
    skcuda = types.ModuleType("skcuda")
    cublas = types.ModuleType("skcuda.cublas")
    cublas.cublasCreate = lambda: 0
    cublas.cublasDestroy = lambda h: None
    cublas.cublasCcopy = _copy(8)
    cublas.cublasZcopy = _copy(16)
    skcuda.cublas = cublas
    mods["skcuda"], mods["skcuda.cublas"] = skcuda, cublas
    hera_cal = types.ModuleType("hera_cal")
    hc_redcal = types.ModuleType("hera_cal.redcal")
    hc_redcal.OmnicalSolver = type("OmnicalSolver", (), {})
    hc_redcal.RedundantCalibrator = type("RedundantCalibrator", (), {})
    hera_cal.redcal = hc_redcal
    mods["hera_cal"], mods["hera_cal.redcal"] = hera_cal, hc_redcal
    linsolve = types.ModuleType("linsolve")
    # linsolve's rule: a trailing '_' marks a conjugated variable and is
    # not part of its name
    linsolve.get_name = lambda s: s.rstrip("_") if isinstance(s, str) else str(s)
    mods["linsolve"] = linsolve
    clash = [k for k in mods if k in sys.modules]
    assert not clash, f"real modules present: {clash}"
    sys.modules.update(mods)
    try:
        yield
    finally:
        for k in mods:
            sys.modules.pop(k, None)


def reference_omnical(ref_root, *args, **kwargs):
    """hera_gpu.redcal.omnical(*args, **kwargs) of the reference sources under
    ref_root, the reference's own code, on the CPU (see the module
    docstring)."""
    with _stubs():
        path = os.path.join(ref_root, "hera_gpu", "redcal.py")
        spec = importlib.util.spec_from_file_location("_reference_redcal", path)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        return mod.omnical(*args, **kwargs)


def reference_solve_iteratively(ref_root, attrs, **kwargs):
    """The reference's ``OmnicalSolverGPU.solve_iteratively``
    (redcal.py:747-837) on an OmnicalSolverGPU whose attributes are
    ``attrs`` (sol0, all_terms, keys, data, wgts, gain), the reference's own
    code on the CPU.  Returns (meta, sol, calls): ``calls`` records the
    arguments and the result of every ``omnical`` call it made."""
    calls = []
    with _stubs():
        path = os.path.join(ref_root, "hera_gpu", "redcal.py")
        spec = importlib.util.spec_from_file_location("_reference_redcal", path)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        inner = mod.omnical

        def recording(*args, **kw):
            out = inner(*args, **kw)
            calls.append({"args": args, "kwargs": kw, "result": out})
            return out

        mod.omnical = recording
        solver = mod.OmnicalSolverGPU()
        solver.__dict__.update(attrs)
        meta, sol = solver.solve_iteratively(**kwargs)
    return meta, sol, calls
