"""Runs CUDA kernels of the reference's sources on the CPU -- TEST
INFRASTRUCTURE ONLY (used by oracle/redcal_ref.py and oracle/median_ref.py).

The reference compiles its kernels at run time from source strings
(pycuda SourceModule).  Here such a string is compiled with g++ behind a
prelude that defines the CUDA built-ins for the host -- blockIdx, threadIdx,
blockDim and gridDim, __shared__ arrays and __global__ / __device__
functions as static ones, the integer min / max, and textures (a
``texture`` object holds a host array set through ``get_texref(name)
.set_array``; ``fp_tex3D`` is an unnormalised, point-sampled, clamped fetch,
the reference's texture set-up) -- into oracle/_ref/.  The source is
compiled as given; nothing of it is rewritten.  Two ways to run a launch:

* sequential (default): every thread of the grid in turn, blocks y-major,
  then the threads of a block y-major; __syncthreads is nothing and
  atomicAdd a plain addition.  Right for kernels whose barriers only order
  writes before reads of later threads in that order.
* barriers: one block at a time, each of its threads a fiber (ucontext)
  on the calling thread; __syncthreads returns to the block's scheduler,
  which runs every thread that has not returned up to its next barrier
  before any goes past it -- CUDA's barrier semantics, deterministic.
  atomicAdd is a plain addition (one thread at a time).  Right for any
  kernel whose threads exchange data through shared memory in both
  directions.
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
#include <cstddef>
#include <texture_types.h>
%(includes)s
#undef __global__
#undef __device__
#define __global__ static
#define __device__ static
typedef unsigned int uint;
struct EmuDim3 { unsigned x, y, z; };
static EmuDim3 blockIdx, blockDim, gridDim;
#define __shared__ static
static inline int min(int a, int b) { return a < b ? a : b; }
static inline int max(int a, int b) { return a > b ? a : b; }
static inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }
static inline unsigned max(unsigned a, unsigned b) { return a > b ? a : b; }
template <typename T, int D = 1, int M = 0> struct texture {
  const T* data = nullptr;
  int w = 0, h = 0, d = 0;
};
typedef float fp_tex_float;
typedef double fp_tex_double;
static inline long emu_texel(double c, int n) {
  long i = (long)std::floor(c);
  return i < 0 ? 0 : (i >= n ? n - 1 : i);
}
template <typename T, int D, int M>
static inline T fp_tex3D(const texture<T, D, M>& t, double x, double y, double z) {
  return t.data[(emu_texel(z, t.d) * t.h + emu_texel(y, t.h)) * t.w + emu_texel(x, t.w)];
}
%(mode)s
"""

SEQUENTIAL = r"""
static EmuDim3 threadIdx;
#define __syncthreads()
static inline float atomicAdd(float* a, float v) { float o = *a; *a = o + v; return o; }
static inline double atomicAdd(double* a, double v) { double o = *a; *a = o + v; return o; }
"""

BARRIERS = r"""
#include <ucontext.h>
#include <functional>
#include <vector>
static EmuDim3 threadIdx;
// Each thread of a block is a fiber (ucontext) on this one OS thread; a
// barrier hands control back to the block's scheduler, which runs every
// live fiber up to its next barrier (or its return) before any goes on.
struct EmuFiber {
  ucontext_t ctx;
  unsigned tx, ty, tz;
  bool done;
};
static ucontext_t emu_main;
static EmuFiber* emu_cur;
static std::function<void()> emu_body;
static void emu_entry() { emu_body(); emu_cur->done = true; }
#define __syncthreads() swapcontext(&emu_cur->ctx, &emu_main)
static void emu_run_block(long nth, unsigned tbx, unsigned tby, std::function<void()> body) {
  const size_t stack = 256 * 1024;
  static std::vector<char> stacks;
  if (stacks.size() < stack * nth) stacks.resize(stack * nth);
  std::vector<EmuFiber> fib((size_t)nth);
  emu_body = std::move(body);
  for (long t = 0; t < nth; ++t) {
    EmuFiber& f = fib[(size_t)t];
    f.tx = (unsigned)(t % tbx); f.ty = (unsigned)(t / tbx % tby); f.tz = (unsigned)(t / tbx / tby);
    f.done = false;
    getcontext(&f.ctx);
    f.ctx.uc_stack.ss_sp = stacks.data() + stack * (size_t)t;
    f.ctx.uc_stack.ss_size = stack;
    f.ctx.uc_link = &emu_main;
    makecontext(&f.ctx, emu_entry, 0);
  }
  for (bool live = true; live;) {
    live = false;
    for (EmuFiber& f : fib) {
      if (f.done) continue;
      emu_cur = &f;
      threadIdx = {f.tx, f.ty, f.tz};
      swapcontext(&emu_main, &f.ctx);
      live |= !f.done;
    }
  }
}
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


def parse_textures(code):
    """Names of the file-scope ``texture<...> name;`` declarations."""
    return re.findall(r"texture\s*<[^;{}]*>\s*(\w+)\s*;", code)


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


class _TexRef:
    """A texture of the module: ``set_array`` points it at a host array of
    shape (depth, height, width), which it keeps alive."""

    def __init__(self, setter):
        self.setter, self.array = setter, None

    def set_array(self, array):
        a = np.ascontiguousarray(array.arr if hasattr(array, "arr") else array)
        d, h, w = (1,) * (3 - a.ndim) + a.shape
        self.array = a
        self.setter(ctypes.c_void_p(a.ctypes.data), w, h, d)


_SEQUENTIAL_LAUNCH = (
    "  for (unsigned y = 0; y < gy; ++y) for (unsigned x = 0; x < gx; ++x) {{\n"
    "    blockIdx = {{x, y, 0u}};\n"
    "    for (unsigned tz = 0; tz < tbz; ++tz) for (unsigned ty = 0; ty < tby; ++ty)\n"
    "      for (unsigned tx = 0; tx < tbx; ++tx) {{\n"
    "        threadIdx = {{tx, ty, tz}}; {name}({call});\n"
    "      }}\n  }}\n")

_BARRIER_LAUNCH = (
    "  const long nth = (long)tbx * tby * tbz;\n"
    "  for (unsigned y = 0; y < gy; ++y) for (unsigned x = 0; x < gx; ++x) {{\n"
    "    blockIdx = {{x, y, 0u}};\n"
    "    emu_run_block(nth, tbx, tby, [&] {{ {name}({call}); }});\n"
    "  }}\n")


class Module:
    """The kernels of one source string, compiled for the host; ``barriers``
    picks how a launch runs its threads (see the module docstring)."""

    def __init__(self, code, includes="", defines="", barriers=False):
        kernels = parse_kernels(code)
        textures = parse_textures(code)
        launch = _BARRIER_LAUNCH if barriers else _SEQUENTIAL_LAUNCH
        wrappers = []
        for name, ps in kernels:
            decl = ", ".join(f"{t} {n}" for _, t, n in ps)
            call = ", ".join(n for _, _, n in ps)
            wrappers.append(
                f'extern "C" void emu_{name}(unsigned gx, unsigned gy, unsigned tbx, unsigned tby, '
                f"unsigned tbz{', ' if decl else ''}{decl}) {{\n"
                "  gridDim = {gx, gy, 1u}; blockDim = {tbx, tby, tbz};\n"
                + launch.format(name=name, call=call) + "}\n")
        for t in textures:
            wrappers.append(
                f'extern "C" void emu_settex_{t}(const void* p, int w, int h, int d) {{\n'
                f"  {t}.data = static_cast<decltype({t}.data)>(p); {t}.w = w; {t}.h = h; "
                f"{t}.d = d;\n}}\n")
        src = defines + PRELUDE % {"includes": includes,
                                   "mode": BARRIERS if barriers else SEQUENTIAL} + \
            code + "\n" + "".join(wrappers)
        key = hashlib.sha256(src.encode()).hexdigest()[:16]
        os.makedirs(OUT, exist_ok=True)
        inc = os.path.join(OUT, "include")
        os.makedirs(inc, exist_ok=True)
        open(os.path.join(inc, "pycuda-helpers.hpp"), "w").close()
        so = os.path.join(OUT, f"kernels_{key}.so")
        if not os.path.exists(so):
            cpp = so[:-3] + ".cpp"
            open(cpp, "w").write(src)
            subprocess.run(["g++", "-std=c++17", "-O2", "-shared", "-fPIC", "-w",
                            "-I", CUDA_INCLUDE, "-I", inc, cpp, "-o", so], check=True)
        lib = ctypes.CDLL(so)
        self.kernels = {name: Kernel(getattr(lib, f"emu_{name}"), ps) for name, ps in kernels}
        self.textures = {}
        for t in textures:
            setter = getattr(lib, f"emu_settex_{t}")
            setter.restype = None
            setter.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
            self.textures[t] = _TexRef(setter)

    def get_function(self, name):
        return self.kernels[name]

    def get_texref(self, name):
        return self.textures[name]
