"""Serving form: continuous batching returns each request's own result.

Requests that arrive close together are served in shared batches on two
slots; every result must equal the result of the same request served alone
(each simulation of a batch keeps its own work items and reduction order),
and agree with the FP64 oracle within the tensor-core tolerance on every
channel and time it asked for.
"""
import numpy as np
import pytest

from hera_gpu_gb300 import _native, serve
from oracle import rel_frobenius, vis_oracle

pytestmark = pytest.mark.gpu


def small_workload(seed=0, n=14):
    specs = [dict(seed=11, nant=20, P=15), dict(seed=12, nant=150, P=31),
             dict(seed=13, nant=300, P=31)]
    rng = np.random.default_rng(seed)
    reqs, t = [], 0.0
    for rid in range(n):
        t += rng.exponential(2e-4)  # 5000 req/s: they pile up into batches
        r = serve.Request(rid, int(rng.integers(3)), int(rng.integers(200, 3000)),
                          int(rng.integers(1, 4)), int(rng.integers(1, 5)), t)
        serve.make_sky(r, seed=int(rng.integers(1 << 30)), lst0=float(rng.uniform(0, 6.28)))
        reqs.append(r)
    return specs, reqs


def test_results_same_alone_and_in_the_mix():
    ctxs = [_native.Context(0), _native.Context(0)]
    specs, reqs = small_workload()
    sets = serve.build_sets(ctxs[0], specs, nfreq=4)
    server = serve.Server(sets, ctxs, hbm_budget=8e9, max_batch=8)
    mixed = server.run(reqs)
    assert all(r.result is not None and r.t_done >= r.arrival for r in mixed)
    stats = serve.summarize(mixed, max(r.t_done for r in mixed))
    assert stats["p99_ms"] >= stats["p50_ms"] > 0
    mixed_results = {r.rid: r.result.copy() for r in mixed}
    # the same requests, one at a time
    alone_server = serve.Server(sets, ctxs[:1], hbm_budget=8e9, max_batch=1)
    for r in reqs:
        r2 = serve.Request(r.rid, r.set_id, r.nsrc, r.ntimes, r.nfreq, 0.0,
                           r.crd_eq, r.I_sky, r.eq2tops)
        alone = alone_server.run([r2])[0].result
        np.testing.assert_array_equal(alone, mixed_results[r.rid])
    for s in sets:
        s.close()


def test_server_matches_oracle():
    ctx = _native.Context(0)
    specs, reqs = small_workload(seed=3, n=4)
    sets = serve.build_sets(ctx, specs, nfreq=4)
    done = serve.Server(sets, [ctx], hbm_budget=8e9, max_batch=4).run(reqs)
    for r in done:
        sp = specs[r.set_id]
        rng = np.random.default_rng(sp["seed"])
        full = serve.synth.hex_array(350, 14.6, 0.01, rng)
        pick = np.sort(rng.choice(350, size=sp["nant"], replace=False))
        dish = 14.0 * (1.0 + 0.02 * rng.uniform(-1.0, 1.0, sp["nant"]))
        assert r.result.shape == (r.nfreq, r.ntimes, sp["nant"], sp["nant"])
        for f in range(r.nfreq):  # every channel of the request, every time
            fq = sets[r.set_id].freqs[f]
            bm = serve.synth.airy_beams(sp["nant"], sp["P"], fq, dish).astype(np.float32)
            ref = vis_oracle(full[pick].astype(np.float32).astype(np.float64), fq,
                             r.eq2tops.astype(np.float64), r.crd_eq.astype(np.float64),
                             r.I_sky.astype(np.float64), bm.astype(np.float64))
            assert rel_frobenius(r.result[f], ref).max() <= 1e-4, (r.rid, f)
    for s in sets:
        s.close()
