"""What the compiler reports for the CUDA sources, with the library's own
flags (``nvcc -Xptxas -v``; it cross-compiles for sm_103a, no GPU is used).

* Every kernel but the fused visibility kernel keeps its values in
  registers: no spills.
* ``tc_vis_kernel`` has eight variants: cluster / one-CTA x batched /
  single simulation x split-BF16 / FP16 + FP8 form.  The split-BF16 form
  runs 15 warps, at most 4 on each of the SM's 4 schedulers, so a thread may
  hold 128 registers, and spills at most 64 bytes; the FP16 + FP8 form runs
  19 warps, so the busiest scheduler holds 5 and a thread 96 registers, and
  spills at most 152 bytes.  A change that spills more would slow the
  latency-bound phasor generators.
"""
import concurrent.futures as cf
import glob
import os
import re
import subprocess

import pytest

from hera_gpu_gb300 import build

ENTRY = re.compile(r"Compiling entry function '(\w+)' for 'sm_103a'.*?"
                   r"(\d+) bytes spill stores, (\d+) bytes spill loads.*?Used (\d+) registers",
                   re.S)


def ptxas_report(src, out_dir):
    obj = os.path.join(out_dir, os.path.basename(src) + ".o")
    p = subprocess.run([build.nvcc(), *build.NVCC_FLAGS, "-Xptxas", "-v", "-c", src, "-o", obj],
                       capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    return {name: (int(st), int(ld), int(regs)) for name, st, ld, regs in ENTRY.findall(p.stderr)}


@pytest.fixture(scope="module")
def reports(tmp_path_factory):
    out = tmp_path_factory.mktemp("ptxas")
    srcs = sorted(glob.glob(os.path.join(build.CSRC, "*.cu")))
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        return dict(zip((os.path.basename(s) for s in srcs),
                        ex.map(lambda s: ptxas_report(s, str(out)), srcs)))


def test_every_source_reports_its_kernels(reports):
    assert set(reports) >= {"hv_tc.cu", "hv_plain.cu", "hv_prep.cu", "hv_omnical.cu",
                            "hv_median.cu", "hv_batch.cu"}
    assert len([k for k in reports["hv_tc.cu"] if "tc_vis_kernel" in k]) == 8


def test_no_kernel_but_the_fused_one_spills(reports):
    spilling = [(src, name, st) for src, r in reports.items() for name, (st, ld, _) in r.items()
                if (st or ld) and "tc_vis_kernel" not in name]
    assert not spilling


def test_fused_kernel_register_budget(reports):
    for name, (stores, loads, regs) in reports["hv_tc.cu"].items():
        if "tc_vis_kernel" in name:
            split_bf16 = "Li0E" in name   # the form template argument, 0 = split BF16
            assert regs <= (128 if split_bf16 else 96), (name, regs)
            assert stores <= (64 if split_bf16 else 152), (name, stores)
