"""The C ABI library: it loads, exports every declared entry point, and the
Python host layer checks shapes like the reference -- all without a GPU."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from hera_gpu_gb300 import _native, vis_gpu
from noalloc_sizes import SCRATCH_BYTES, largest_nsrc, need_bytes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(hv_[a-z0-9_]+)\s*\(", text))
    return names


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_native.LIB_PATH):
        from hera_gpu_gb300 import build
        build.build()
    return _native.load_library()


def test_library_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert {"hv_create", "hv_destroy", "hv_vis_gpu", "hv_vis_multifreq",
            "hv_vis_multifreq_device", "hv_last_error", "hv_sync"} <= names
    out = subprocess.run(["nm", "-D", "--defined-only", _native.LIB_PATH],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (hv_[a-z0-9_]+)", out))
    assert names <= exported, names - exported
    for n in names:
        assert hasattr(lib, n)
    assert set(_native.SIGNATURES) == names


def test_version(lib):
    assert lib.hv_version() >= 10000


def test_create_without_gpu_fails_loudly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(_native.HeraVisError):
        _native.Context(0)


NANT, NTIMES, BM_PIX, NPIX = 16, 10, 31, 12 * 16 ** 2


@pytest.mark.parametrize("bad", ["antpos", "eq2tops", "crd_eq", "bm_cube", "I_sky"])
def test_shape_asserts_before_any_device_work(bad):
    # test_vis_gpu.py:172-191 of the reference: transposed inputs raise AssertionError
    args = dict(antpos=np.zeros((NANT, 3)), eq2tops=np.zeros((NTIMES, 3, 3)),
                crd_eq=np.zeros((3, NPIX)), I_sky=np.zeros(NPIX),
                bm_cube=np.zeros((NANT, BM_PIX, BM_PIX)))
    if bad == "I_sky":
        args[bad] = np.zeros((NPIX, 1))
    else:
        args[bad] = args[bad].T
    with pytest.raises(AssertionError):
        vis_gpu(args["antpos"], 0.15, args["eq2tops"], args["crd_eq"], args["I_sky"],
                args["bm_cube"])


def test_precision_must_be_1_or_2():
    with pytest.raises(AssertionError):
        vis_gpu(np.zeros((2, 3)), 0.15, np.zeros((1, 3, 3)), np.zeros((3, 4)), np.zeros(4),
                np.zeros((2, 3, 3)), precision=3)


def test_omnical_asserts_before_any_device_work():
    # redcal.py:392-402 of the reference
    from hera_gpu_gb300 import omnical
    ggu = np.array([(1, 0, 0)], dtype=np.uint32)
    g, u, d, w = np.ones((2, 2)), np.ones((2, 1)), np.ones((2, 1)), np.ones((2, 1))
    for kw in (dict(ggu_indices=ggu.T), dict(check_every=1), dict(precision=3),
               dict(data=np.ones((2, 2))), dict(wgts=np.ones((3, 1))), dict(ubls=np.ones(2))):
        args = dict(ggu_indices=ggu, gains=g, ubls=u, data=d, wgts=w)
        extra = {k: v for k, v in kw.items() if k not in args}
        args.update({k: v for k, v in kw.items() if k in args})
        with pytest.raises((AssertionError, IndexError)):
            omnical(**args, **extra)


def test_median_filter_asserts_before_any_device_work():
    from hera_gpu_gb300 import MedianFilter
    with pytest.raises(AssertionError):
        MedianFilter(input=np.zeros((4, 4)), kernel_size=0)
    with pytest.raises(AssertionError):
        MedianFilter(input=np.zeros(4), kernel_size=3)


def test_entry_points_reject_a_null_context(lib):
    # HV_ERR_ARG (1), checked before any CUDA call
    ARG = 1
    d, u, p = ctypes.c_double(), ctypes.c_uint64(), ctypes.c_void_p()
    assert lib.hv_create(None, 0, 0) == ARG
    assert lib.hv_vis_gpu(None, 1, 0, None, 4, 1e8, None, 1, None, None, 1, None, 3, None) == ARG
    assert lib.hv_vis_multifreq(None, 1, 0, None, 4, None, 1, None, 1, None, None, 1, None, 3,
                                None) == ARG
    assert lib.hv_vis_multifreq_device(None, 1, 0, None, 4, None, 1, None, 1, None, None, 1, None,
                                       3, None, None) == ARG
    assert lib.hv_sync(None) == ARG
    assert lib.hv_set_profiling(None, 1) == ARG
    assert lib.hv_profile_read(None, ctypes.byref(d), ctypes.byref(u)) == ARG
    assert lib.hv_set_wait_limit(None, 0, 0) == ARG
    assert lib.hv_set_tuning(None, 2, 0) == ARG
    assert lib.hv_device_alloc(None, 16, ctypes.byref(p)) == ARG
    assert lib.hv_device_free(None, None) == ARG
    assert lib.hv_memcpy_async(None, None, None, 0, 1) == ARG
    assert lib.hv_stream_query(None) == -ARG
    assert lib.hv_host_alloc(None, 16, ctypes.byref(p)) == ARG
    assert lib.hv_host_free(None, None) == ARG
    assert lib.hv_batch_create(None, None, 1, 0, ctypes.byref(p)) == ARG
    assert lib.hv_batch_launch(None, None) == ARG
    assert lib.hv_batch_sync(None) == ARG
    assert lib.hv_vis_batch(None, None, 1, None) == ARG
    assert lib.hv_omnical(None, 1, None, 0, None, 0, None, 0, None, None, 0, 1e-10, 50, 4, 1,
                          0.3, None, None, None) == ARG
    assert lib.hv_omnical_device(None, 1, None, 0, None, 0, None, 0, None, None, 0, 1e-10, 50,
                                 4, 1, 0.3, None, None, None, None) == ARG
    assert lib.hv_median_filter(None, None, None, 0, 0, 0, 3, 3) == ARG
    assert lib.hv_median_filter_device(None, None, None, 0, 0, 0, 3, 3, None) == ARG
    # nothing to release, nothing counted
    assert lib.hv_destroy(None) == 0 and lib.hv_batch_destroy(None) == 0
    assert lib.hv_launch_count(None) == 0 and lib.hv_batch_launches(None) == 0
    assert lib.hv_last_error(None) == b"no context"


def test_noalloc_entry_point_checks_arguments_first(lib):
    # hv_vis_gpu_noalloc has no context: its errors come back in errbuf
    buf = ctypes.create_string_buffer(256)
    assert lib.hv_vis_gpu_noalloc(None, 0, 1e8, None, 1, None, None, 1, None, 3, None, None, buf,
                                  len(buf)) == 1
    assert b"bad sizes" in buf.value
    assert lib.hv_vis_gpu_noalloc(None, 4, 1e8, None, 1, None, None, 1, None, 3, None, None, buf,
                                  len(buf)) == 1
    assert b"null array argument" in buf.value
    # the antenna limit of the allocating entry points, before any size is formed
    for nant in (65537, 2**31 - 1):
        assert lib.hv_vis_gpu_noalloc(None, nant, 1e8, None, 1, None, None, 1, None, 3, None, None,
                                      buf, len(buf)) == 1
        assert b"bad sizes" in buf.value


def test_noalloc_refuses_one_source_past_its_array(lib):
    # a request one source past the largest that fits is refused by the size
    # check, which comes before any CUDA call (the pointers are never read)
    nant, ntimes, P = 150, 2, 31
    nsrc = largest_nsrc(nant, ntimes, P)
    assert need_bytes(nant, nsrc + 1, ntimes, P) > SCRATCH_BYTES
    buf = ctypes.create_string_buffer(512)
    one = ctypes.c_void_p(1)
    assert lib.hv_vis_gpu_noalloc(one, nant, 1e8, one, ntimes, one, one, nsrc + 1, one, P, one,
                                  None, buf, len(buf)) == 1
    assert b"working memory" in buf.value
    assert str(need_bytes(nant, nsrc + 1, ntimes, P)).encode() in buf.value


@pytest.mark.parametrize("std", ["c99", "c11"])
def test_header_is_plain_c(tmp_path, std):
    # the boundary is a C ABI: the header compiles as C, pedantic, warnings as errors
    src = tmp_path / "use.c"
    src.write_text('#include "heravis.h"\nint main(void) { hv_context* c = 0; (void)c; return 0; }\n')
    subprocess.run(["gcc", f"-std={std}", "-Wall", "-Wextra", "-pedantic", "-Werror",
                    "-fsyntax-only", "-I", os.path.join(ROOT, "include"), str(src)], check=True)


def test_status_codes_map_to_exceptions(lib):
    # a Context with no device behind it: only the status -> exception mapping runs
    ctx = _native.Context.__new__(_native.Context)
    ctx.lib, ctx.h = lib, None
    ctx.check(_native.HV_OK)
    # bad arguments raise AssertionError, as the reference's asserts do
    with pytest.raises(AssertionError) as e:
        ctx.check(1)
    assert isinstance(e.value, _native.HeraVisArgumentError) and e.value.code == 1
    assert "no context" in str(e.value)
    with pytest.raises(_native.HeraVisTimeout):
        ctx.check(4)
    for code in (2, 3, 5):
        with pytest.raises(_native.HeraVisError) as e:
            ctx.check(code)
        assert type(e.value) is _native.HeraVisError and e.value.code == code


def header_enum(name):
    text = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "heravis.h")).read(),
                  flags=re.S)
    return int(re.search(rf"\b{name}\s*=\s*(\d+)", text).group(1))


def test_python_constants_match_the_header():
    for name in ("HV_OK", "HV_ERR_ARG", "HV_ERR_OOM", "HV_ERR_CUDA", "HV_ERR_TIMEOUT",
                 "HV_ERR_UNSUPPORTED", "HV_BATCH_GRAPH", "HV_BATCH_AUTOTUNE"):
        assert getattr(_native, name) == header_enum(name), name
    assert _native.METHODS["auto"] == header_enum("HV_METHOD_AUTO")
    assert _native.METHODS["plain"] == header_enum("HV_METHOD_PLAIN")
    assert _native.METHODS["tc"] == _native.METHODS["tc_bf16"] == header_enum("HV_METHOD_TC_BF16")
    assert _native.METHODS["tc_fp16"] == header_enum("HV_METHOD_TC_FP16")
    assert _native.HV_TUNE_STAGES == header_enum("HV_TUNE_STAGES")


def test_hv_sim_layout_matches_the_header(tmp_path):
    # the C compiler's layout of hv_sim against the ctypes mirror
    fields = [f for f, _ in _native.HvSim._fields_]
    src = tmp_path / "layout.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "heravis.h"\nint main(void) {\n'
                   '  printf("%zu\\n", sizeof(hv_sim));\n'
                   + "".join(f'  printf("%zu\\n", offsetof(hv_sim, {f}));\n' for f in fields)
                   + "  return 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    assert got[0] == ctypes.sizeof(_native.HvSim)
    assert got[1:] == [getattr(_native.HvSim, f).offset for f in fields]


def _c_kind(decl):
    decl = " ".join(decl.split())
    if "*" in decl:
        return "ptr"
    for word, kind in (("double", "f64"), ("uint64_t", "u64"), ("size_t", "u64"),
                       ("unsigned", "u32"), ("int", "i32")):
        if re.search(rf"\b{word}\b", decl):
            return kind
    raise ValueError(decl)


def _ctypes_kind(t):
    if t in (ctypes.c_void_p, ctypes.c_char_p) or (isinstance(t, type) and
                                                    issubclass(t, ctypes._Pointer)):
        return "ptr"
    if t is ctypes.c_double:
        return "f64"
    if t in (ctypes.c_size_t, ctypes.c_uint64):
        return "u64"
    if t is ctypes.c_uint:
        return "u32"
    if t is ctypes.c_int:
        return "i32"
    raise ValueError(t)


def test_ctypes_signatures_match_the_header_prototypes():
    text = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "heravis.h")).read(),
                  flags=re.S)
    protos = re.findall(r"([A-Za-z_][\w\s\*]*?)\b(hv_\w+)\s*\(([^)]*)\)\s*;", text)
    assert {name for _, name, _ in protos} == set(_native.SIGNATURES)
    for ret, name, params in protos:
        res, args = _native.SIGNATURES[name]
        params = [] if params.strip() in ("", "void") else params.split(",")
        assert [_c_kind(p) for p in params] == [_ctypes_kind(a) for a in args], name
        assert _c_kind(ret) == _ctypes_kind(res), name


def test_integration_guide_binding_matches_the_header():
    # the ctypes binding INTEGRATION.md shows a maintainer of the reference
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    code = re.search(r"```python\nimport ctypes, numpy as np\n(.*?)```", doc, re.S).group(1)
    for name in ("hv_create", "hv_vis_gpu"):
        listed = re.search(rf"_lib\.{name}\.argtypes = (\[.*?\])", code, re.S).group(1)
        args = eval(listed, {"ctypes": ctypes})
        assert [_ctypes_kind(a) for a in args] == \
            [_ctypes_kind(a) for a in _native.SIGNATURES[name][1]], name


@pytest.mark.parametrize("kwargs,want", [
    ({}, 1),
    ({"precision": 2}, 2),
    ({"real_dtype": np.float64}, 2),
    ({"real_dtype": np.float32}, 1),
    ({"complex_dtype": np.complex128}, 2),
    ({"real_dtype": np.float64, "complex_dtype": np.complex128}, 2),
    ({"precision": 1, "real_dtype": np.float32, "complex_dtype": np.complex64}, 1),
])
def test_precision_spellings(kwargs, want):
    # the reference's precision (vis.py:147-157) and vis_cpu's dtype spelling
    from hera_gpu_gb300.vis import _resolve_precision
    args = {"precision": None, "real_dtype": None, "complex_dtype": None}
    args.update(kwargs)
    p, rt, ct = _resolve_precision(args["precision"], args["real_dtype"], args["complex_dtype"])
    assert p == want
    assert (rt, ct) == ((np.float32, np.complex64) if want == 1 else (np.float64, np.complex128))


@pytest.mark.parametrize("kwargs", [
    {"precision": 3},
    {"precision": 1, "real_dtype": np.float64},
    {"precision": 2, "complex_dtype": np.complex64},
    {"real_dtype": np.float64, "complex_dtype": np.complex64},
])
def test_conflicting_precision_spellings_raise(kwargs):
    from hera_gpu_gb300.vis import _resolve_precision
    args = {"precision": None, "real_dtype": None, "complex_dtype": None}
    args.update(kwargs)
    with pytest.raises(AssertionError):
        _resolve_precision(args["precision"], args["real_dtype"], args["complex_dtype"])


def test_positional_nthreads_of_a_reference_caller_is_an_assertion():
    # the reference takes nthreads at position 7 (vis.py:144-146); here that
    # position is real_dtype, so an integer there is refused as the
    # reference refuses bad arguments, before any device work
    with pytest.raises(AssertionError, match="keyword"):
        vis_gpu(np.zeros((2, 3)), 1e8, np.zeros((1, 3, 3)), np.zeros((3, 4)), np.zeros(4),
                np.zeros((2, 3, 3)), 1024)
