"""The reference's own vis_gpu, run on the CPU -- TEST INFRASTRUCTURE ONLY.

Runs the unmodified ``vis_gpu`` of hera_gpu/vis.py:144-262 (its chunking,
its stream loop and its host-side sum) and its two CUDA kernels,
``InterpolateBeam`` and ``MeasEq`` (the GPU_TEMPLATE string, vis.py:10-111),
without a GPU, to produce reference outputs for tests/golden/
(make_vis_gpu_golden.py):

* ``SourceModule`` is oracle/cuda_emu.py with barriers: the kernel source
  exactly as the reference formats it, compiled with g++ for the host, each
  block's threads run as fibers that all reach a barrier before any passes
  it, since InterpolateBeam's threads exchange beam coordinates through
  shared memory in both directions.  CUDA's float overloads of cos / sin /
  fma are the C++ library's float overloads.
* The beam texture is a host array read by point-sampled, clamped fetches
  at unnormalised coordinates -- the reference's texture set-up
  (vis.py:113-138: an array of (nant, P, P), no filtering, default address
  mode).
* cuBLAS's four GEMMs (vis.py:228-249) are numpy matrix products in the
  same precision with cuBLAS's column-major argument convention; their
  summation order is BLAS's, not cuBLAS's.
* pycuda arrays are numpy arrays (zero-filled), streams and events do
  nothing, and astropy's ``c`` is 299792458 m/s.

Launches run in program order, so each chunk's kernels see that chunk's
sources, as the reference intends.  Needs the reference sources; the tests
use the fixtures it made.
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

_INCLUDES = """#include <cuComplex.h>
using std::cos;
using std::sin;
using std::fma;
"""


class _GPUArray:
    def __init__(self, shape, dtype):
        self.arr = np.zeros(shape, dtype=dtype)
        self.gpudata = self.arr.ctypes.data

    def set(self, a):
        self.arr[...] = a

    def set_async(self, a, stream=None):
        self.arr[...] = a

    def get_async(self, ary=None, stream=None):
        if ary is None:
            return self.arr.copy()
        np.copyto(ary, self.arr)
        return ary


def _to_gpu(a):
    g = _GPUArray(a.shape, a.dtype)
    g.set(a)
    return g


class _Stream:
    handle = 0


class _Event:
    def record(self, stream=None):
        pass

    def synchronize(self):
        pass


class _Bag:
    """An attribute holder (ArrayDescriptor3D, Memcpy3D settings)."""


class _Array:
    def __init__(self, descr):
        self.descr, self.arr = descr, None


class _Memcpy3D(_Bag):
    def set_src_host(self, a):
        self.src = a

    def set_dst_array(self, dst):
        self.dst = dst

    def __call__(self):
        self.dst.arr = np.ascontiguousarray(self.src)


def _source_module(code):
    return cuda_emu.Module(code, includes=_INCLUDES, barriers=True)


def _gemm(dtype):
    dtype = np.dtype(dtype)

    def mat(ptr, rows, cols, ld):
        # a column-major rows x cols matrix with leading dimension ld
        buf = (ctypes.c_char * (ld * cols * dtype.itemsize)).from_address(int(ptr))
        return np.frombuffer(buf, dtype=dtype).reshape(cols, ld)[:, :rows].T

    def op(x, trans):
        return x if trans == "n" else (x.T if trans == "t" else x.conj().T)

    def gemm(handle, transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc):
        a = op(mat(A, m, k, lda) if transa == "n" else mat(A, k, m, lda), transa)
        b = op(mat(B, k, n, ldb) if transb == "n" else mat(B, n, k, ldb), transb)
        c = mat(C, m, n, ldc)
        r = dtype.type(alpha) * (a @ b)
        if beta != 0:
            r = r + dtype.type(beta) * c
        c[...] = r.astype(dtype)

    return gemm


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
    mods["pycuda.gpuarray"].to_gpu = _to_gpu
    drv = mods["pycuda.driver"]
    drv.Stream, drv.Event, drv.Array, drv.Memcpy3D = _Stream, _Event, _Array, _Memcpy3D
    drv.ArrayDescriptor3D = _Bag
    drv.array_format = types.SimpleNamespace(SIGNED_INT32="SIGNED_INT32")
    drv.dtype_to_array_format = lambda dt: np.dtype(dt).name
    skcuda = types.ModuleType("skcuda")
    cublas = types.ModuleType("skcuda.cublas")
    cublas.cublasCreate = lambda: 0
    cublas.cublasDestroy = lambda h: None
    cublas.cublasSetStream = lambda h, s: None
    cublas.cublasSgemm = _gemm(np.float32)
    cublas.cublasDgemm = _gemm(np.float64)
    cublas.cublasCgemm = _gemm(np.complex64)
    cublas.cublasZgemm = _gemm(np.complex128)
    skcuda.cublas = cublas
    mods["skcuda"], mods["skcuda.cublas"] = skcuda, cublas
    astropy = types.ModuleType("astropy")
    constants = types.ModuleType("astropy.constants")
    constants.c = types.SimpleNamespace(value=299792458.0)
    astropy.constants = constants
    mods["astropy"], mods["astropy.constants"] = astropy, constants
    clash = [k for k in mods if k in sys.modules]
    assert not clash, f"real modules present: {clash}"
    sys.modules.update(mods)
    try:
        yield
    finally:
        for k in mods:
            sys.modules.pop(k, None)


def reference_vis_gpu(ref_root, *args, **kwargs):
    """hera_gpu.vis.vis_gpu(*args, **kwargs) of the reference sources under
    ref_root, the reference's own code, on the CPU (see the module
    docstring)."""
    with _stubs():
        path = os.path.join(ref_root, "hera_gpu", "vis.py")
        spec = importlib.util.spec_from_file_location("_reference_vis", path)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        return mod.vis_gpu(*args, **kwargs)


def sources_used(nant, nsrc, max_memory=2 ** 29, min_chunk=8):
    """How many sources the reference's vis_gpu sums: it splits them into
    ``chunk`` pieces of ``nsrc // chunk`` and drops the rest (vis.py:176-177)."""
    chunk = max(min(nsrc, min_chunk),
                2 ** int(np.ceil(np.log2(float(nant * nsrc) / max_memory / 2))))
    return (nsrc // chunk) * chunk
