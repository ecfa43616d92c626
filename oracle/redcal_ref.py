"""The reference's own omnical, run on the CPU -- TEST INFRASTRUCTURE ONLY.

Runs the unmodified ``omnical`` of hera_gpu/redcal.py:358-743 (its host loop)
and its CUDA kernels (the GPU_TEMPLATE string, redcal.py:19-355) without a
GPU, to produce reference outputs for tests/golden/ (make_omnical_golden.py):

* the reference's imports are stubbed: pycuda arrays are numpy arrays
  (zero-filled, where pycuda's gpuarray.empty leaves memory as it finds it),
  events are no-ops, the two cuBLAS copies are memory copies, and the
  hera_cal / linsolve names its wrapper classes use are placeholders;
* ``SourceModule`` formats nothing itself: it takes the kernel source exactly
  as the reference formats it, adds a prelude that defines the CUDA
  built-ins for the host (blockIdx / threadIdx as globals, atomicAdd as a
  plain addition, __syncthreads as nothing), compiles it with g++ into
  oracle/_ref/, and runs a launch as a loop over every thread -- blocks
  y-major, then threads y-major, so that in update_active (redcal.py:314-354)
  the thread with td == 0 of a pixel runs before the others that read the
  flag it writes, as the kernel's barrier orders them.

The atomic sums are thus taken in thread order, which the GPU does not fix;
their rounding differs from any one GPU run at the last bits.  Needs the
reference sources; the tests use the fixtures it made.
"""
from __future__ import annotations

import contextlib
import ctypes
import hashlib
import importlib.util
import os
import re
import subprocess
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
CUDA_INCLUDE = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")

PRELUDE = r"""
#define __CUDA_ARCH__ 800  /* skips the template's atomicAdd(double) shim */
#include <cmath>
#include <cstdio>
#include <cuComplex.h>
#undef __global__
#define __global__ static
typedef unsigned int uint;
struct EmuDim3 { unsigned x, y, z; };
static EmuDim3 blockIdx, threadIdx, blockDim, gridDim;
#define __syncthreads()
static inline float atomicAdd(float* a, float v) { float o = *a; *a = o + v; return o; }
static inline double atomicAdd(double* a, double v) { double o = *a; *a = o + v; return o; }
"""

_SCALAR = {"uint": ctypes.c_uint, "float": ctypes.c_float, "double": ctypes.c_double}


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


def _parse_kernels(code):
    """[(name, [(scalar type or None for a pointer, declared type, name)])] of
    every kernel of the formatted template."""
    out = []
    for name, params in re.findall(r"__global__\s+void\s+(\w+)\s*\(([^)]*)\)", code, re.S):
        ps = []
        for p in params.split(","):
            p = " ".join(p.split())
            pname = re.findall(r"(\w+)\s*$", p)[0]
            ptype = p[: -len(pname)].strip()
            ps.append((None if "*" in ptype else ptype, ptype, pname))
        out.append((name, ps))
    return out


class _Kernel:
    def __init__(self, fn, params):
        self.fn, self.params = fn, params
        fn.restype = None
        fn.argtypes = [ctypes.c_uint] * 5 + [ctypes.c_void_p if s is None else _SCALAR[s]
                                             for s, _, _ in params]

    def __call__(self, *args, block, grid):
        conv = []
        for (s, _, _), a in zip(self.params, args):
            if s is None:
                conv.append(ctypes.c_void_p(a.arr.ctypes.data))
            else:
                conv.append(_SCALAR[s](a.item() if hasattr(a, "item") else a))
        gx, gy = (tuple(grid) + (1, 1))[:2]
        bx, by, bz = (tuple(block) + (1, 1, 1))[:3]
        self.fn(gx, gy, bx, by, bz, *conv)


class _SourceModule:
    def __init__(self, code):
        kernels = _parse_kernels(code)
        wrappers = []
        for name, ps in kernels:
            decl = ", ".join(f"{t} {n}" for _, t, n in ps)
            call = ", ".join(n for _, _, n in ps)
            wrappers.append(
                f'extern "C" void emu_{name}(unsigned gx, unsigned gy, unsigned tbx, unsigned tby, '
                f"unsigned tbz{', ' if decl else ''}{decl}) {{\n"
                "  gridDim = {gx, gy, 1u}; blockDim = {tbx, tby, tbz};\n"
                "  for (unsigned y = 0; y < gy; ++y) for (unsigned x = 0; x < gx; ++x) {\n"
                "    blockIdx = {x, y, 0u};\n"
                "    for (unsigned tz = 0; tz < tbz; ++tz) for (unsigned ty = 0; ty < tby; ++ty)\n"
                "      for (unsigned tx = 0; tx < tbx; ++tx) {\n"
                f"        threadIdx = {{tx, ty, tz}}; {name}({call});\n"
                "      }\n  }\n}\n")
        src = PRELUDE + code + "\n" + "".join(wrappers)
        key = hashlib.sha256(src.encode()).hexdigest()[:16]
        os.makedirs(OUT, exist_ok=True)
        inc = os.path.join(OUT, "include")
        os.makedirs(inc, exist_ok=True)
        open(os.path.join(inc, "pycuda-helpers.hpp"), "w").close()
        so = os.path.join(OUT, f"redcal_kernels_{key}.so")
        if not os.path.exists(so):
            cpp = so[:-3] + ".cpp"
            open(cpp, "w").write(src)
            subprocess.run(["g++", "-O2", "-shared", "-fPIC", "-w", "-I", CUDA_INCLUDE, "-I", inc,
                            cpp, "-o", so], check=True)
        lib = ctypes.CDLL(so)
        self.kernels = {name: _Kernel(getattr(lib, f"emu_{name}"), ps) for name, ps in kernels}

    def get_function(self, name):
        return self.kernels[name]


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
    mods["pycuda.compiler"].SourceModule = _SourceModule
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
    linsolve.get_name = lambda s: s
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
