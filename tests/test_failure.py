"""Failure detection on the GPU, without faulting it.

The reference checks only shapes (hera_gpu/vis.py:147,161-169).  Here every
device-side wait of the fused kernel is bounded: a test injects a stall (the
kernel's first source copy is never issued, so the waits on it run out), the
call must come back with a timeout status within the shortened limit, and
the same context must then give the normal result.  The HBM budget of a
context turns an oversized workspace into an out-of-memory status, and the
serving loop keeps serving when one of its slots fails.
"""
import time

import numpy as np
import pytest

from hera_gpu_gb300 import _native, serve, synth, vis_gpu_multifreq

pytestmark = pytest.mark.gpu


def config(nant, nsrc, ntimes=2, nfreq=2, seed=5):
    cfg = synth.config_array(seed=seed, nant=nant, nsrc=nsrc, ntimes=ntimes, nfreq=nfreq,
                             fmin=100e6, fmax=200e6, P=31)
    bm = synth.beams_for(cfg, dtype=np.float32)
    return (cfg["antpos"].astype(np.float32), cfg["freqs"], cfg["eq2tops"].astype(np.float32),
            cfg["crd_eq"].astype(np.float32), cfg["I_sky"].astype(np.float32), bm)


@pytest.mark.parametrize("method", ["tc", "tc_fp16"])
@pytest.mark.parametrize("nant", [40, 300])  # one CTA per item; a cluster of three
def test_injected_stall_times_out_and_context_recovers(nant, method):
    args = config(nant, 3000)
    ctx = _native.Context(0)
    ref = vis_gpu_multifreq(*args, precision=1, method=method, context=ctx)
    ctx.set_wait_limit(0.05, stall=True)
    t0 = time.perf_counter()
    with pytest.raises(_native.HeraVisTimeout):
        vis_gpu_multifreq(*args, precision=1, method=method, context=ctx)
    assert time.perf_counter() - t0 < 30.0
    ctx.set_wait_limit(0.0, stall=False)
    again = vis_gpu_multifreq(*args, precision=1, method=method, context=ctx)
    np.testing.assert_array_equal(again, ref)


def test_hbm_budget_turns_into_out_of_memory():
    args = config(150, 20000)
    small = _native.Context(0, hbm_budget_bytes=1 << 20)
    with pytest.raises(_native.HeraVisError) as e:
        vis_gpu_multifreq(*args, precision=1, method="tc", context=small)
    assert e.value.code == _native.HV_ERR_OOM
    out = vis_gpu_multifreq(*args, precision=1, method="tc", context=_native.Context(0))
    assert np.isfinite(out).all()


def test_serving_continues_when_a_slot_times_out():
    ctxs = [_native.Context(0), _native.Context(0)]
    specs = [dict(seed=21, nant=30, P=15), dict(seed=22, nant=140, P=15)]
    sets = serve.build_sets(ctxs[0], specs, nfreq=2)
    rng = np.random.default_rng(1)
    reqs = []
    for rid in range(8):
        r = serve.Request(rid, rid % 2, int(rng.integers(500, 2000)), 2, 2, 0.0)
        reqs.append(serve.make_sky(r, seed=rid, lst0=0.3 * rid))
    # requests arriving together fill slot 0 first, then slot 1; slot 1 stalls
    ctxs[1].set_wait_limit(0.05, stall=True)
    done = serve.Server(sets, ctxs, hbm_budget=8e9, max_batch=4).run(reqs)
    failed = [r for r in done if r.error]
    served = [r for r in done if r.ok]
    assert failed and served
    assert all("batch failed" in r.error for r in failed)
    # the served results are the ones the same requests give on a healthy slot
    ctxs[1].set_wait_limit(0.0, stall=False)
    for r in served:
        again = serve.Server(sets, ctxs[1:], hbm_budget=8e9, max_batch=1).run(
            [serve.Request(r.rid, r.set_id, r.nsrc, r.ntimes, r.nfreq, 0.0, r.crd_eq, r.I_sky,
                           r.eq2tops)])[0]
        np.testing.assert_array_equal(again.result, r.result)
    for s in sets:
        s.close()
