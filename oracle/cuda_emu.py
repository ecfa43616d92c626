"""Runs CUDA kernels of the reference's sources on the CPU -- TEST
INFRASTRUCTURE ONLY (used by oracle/redcal_ref.py and oracle/median_ref.py).

The reference compiles its kernels at run time from source strings
(pycuda SourceModule).  Here such a string is compiled with g++ behind a
prelude that defines the CUDA built-ins for the host -- blockIdx, threadIdx,
blockDim and gridDim as globals, atomicAdd as a plain addition,
__syncthreads as nothing, __shared__ arrays and __global__ / __device__
functions as static ones, the integer min / max, and an empty ``texture``
template -- into oracle/_ref/.  A launch runs every
thread of the grid in turn: blocks y-major, then the threads of a block
y-major.  The source is compiled as given; nothing of it is rewritten.
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import re
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
CUDA_INCLUDE = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")

PRELUDE = r"""
#include <cmath>
#include <cstdio>
%(includes)s
#undef __global__
#undef __device__
#define __global__ static
#define __device__ static
template <typename T, int D> struct texture {};
typedef unsigned int uint;
struct EmuDim3 { unsigned x, y, z; };
static EmuDim3 blockIdx, threadIdx, blockDim, gridDim;
#define __syncthreads()
#define __shared__ static
static inline int min(int a, int b) { return a < b ? a : b; }
static inline int max(int a, int b) { return a > b ? a : b; }
static inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }
static inline unsigned max(unsigned a, unsigned b) { return a > b ? a : b; }
static inline float atomicAdd(float* a, float v) { float o = *a; *a = o + v; return o; }
static inline double atomicAdd(double* a, double v) { double o = *a; *a = o + v; return o; }
"""

_SCALAR = {"uint": ctypes.c_uint, "int": ctypes.c_int, "float": ctypes.c_float,
           "double": ctypes.c_double}


def parse_kernels(code):
    """[(name, [(scalar type or None for a pointer, declared type, name)])] of
    every __global__ function of the source."""
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


def _address(a):
    if hasattr(a, "arr"):
        a = a.arr
    if isinstance(a, np.ndarray):
        return ctypes.c_void_p(a.ctypes.data)
    return ctypes.c_void_p(int(a))


class Kernel:
    """One kernel: call it as pycuda does (``k(*args, block=, grid=)``), or
    through ``prepare`` / ``prepared_async_call``."""

    def __init__(self, fn, params):
        self.fn, self.params = fn, params
        fn.restype = None
        fn.argtypes = [ctypes.c_uint] * 5 + [ctypes.c_void_p if s is None else _SCALAR[s]
                                             for s, _, _ in params]

    def __call__(self, *args, block, grid, stream=None):
        conv = []
        for (s, _, _), a in zip(self.params, args):
            conv.append(_address(a) if s is None else
                        _SCALAR[s](a.item() if hasattr(a, "item") else a))
        gx, gy = (tuple(grid) + (1, 1))[:2]
        bx, by, bz = (tuple(block) + (1, 1, 1))[:3]
        self.fn(gx, gy, bx, by, bz, *conv)

    def prepare(self, fmt):
        return self

    def prepared_async_call(self, grid, block, stream, *args):
        self(*args, block=block, grid=grid)


class Module:
    """The kernels of one source string, compiled for the host."""

    def __init__(self, code, includes="", defines=""):
        kernels = parse_kernels(code)
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
        src = defines + PRELUDE % {"includes": includes} + code + "\n" + "".join(wrappers)
        key = hashlib.sha256(src.encode()).hexdigest()[:16]
        os.makedirs(OUT, exist_ok=True)
        inc = os.path.join(OUT, "include")
        os.makedirs(inc, exist_ok=True)
        open(os.path.join(inc, "pycuda-helpers.hpp"), "w").close()
        so = os.path.join(OUT, f"kernels_{key}.so")
        if not os.path.exists(so):
            cpp = so[:-3] + ".cpp"
            open(cpp, "w").write(src)
            subprocess.run(["g++", "-O2", "-shared", "-fPIC", "-w", "-I", CUDA_INCLUDE, "-I", inc,
                            cpp, "-o", so], check=True)
        lib = ctypes.CDLL(so)
        self.kernels = {name: Kernel(getattr(lib, f"emu_{name}"), ps) for name, ps in kernels}

    def get_function(self, name):
        return self.kernels[name]

    def get_texref(self, name):
        return None
