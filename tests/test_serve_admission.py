"""Serving loop on the host: admission by HBM budget, cancellation and
failure isolation, with a fake device (no GPU).

The reference has no serving layer (it answers one vis_gpu call at a time,
hera_gpu/vis.py:144); these tests pin the failure behaviour of the loop:
a request larger than the budget is rejected, a cancelled request is never
launched, and a batch that fails (a launch error or a device-side timeout)
fails only its own requests while the loop keeps serving.
"""
import os
import re
import types

import numpy as np
import pytest

from hera_gpu_gb300 import _native, serve


class FakeContext:
    """Host stand-in for a context: pinned buffers are plain arrays, device
    pointers are counters, the stream is always idle."""

    def __init__(self):
        self.next_ptr = 1 << 20
        self.live = {}

    def pinned_empty(self, shape, dtype):
        return np.zeros(shape, dtype)

    def device_alloc(self, nbytes):
        self.next_ptr += max(int(nbytes), 1) + 256
        self.live[self.next_ptr] = nbytes
        return self.next_ptr

    def device_free(self, ptr):
        del self.live[ptr]

    def h2d(self, dst, src):
        pass

    def d2h(self, dst, src):
        dst[...] = 1.0

    def idle(self):
        return True

    def sync(self):
        pass


class FakeBatch:
    """Fails at launch when a simulation has nsrc == 13, at sync (a
    device-side timeout) when one has nsrc == 17."""

    launched = []

    def __init__(self, ctx, sims):
        self.sims = sims

    def launch(self):
        if any(s["nsrc"] == 13 for s in self.sims):
            raise _native.HeraVisError(_native.HV_ERR_OOM, "injected launch failure")
        FakeBatch.launched.extend(s["nsrc"] for s in self.sims)

    def sync(self):
        if any(s["nsrc"] == 17 for s in self.sims):
            raise _native.HeraVisTimeout(_native.HV_ERR_TIMEOUT, "injected device timeout")

    def close(self):
        pass


def fake_sets(n=2, nant=20, P=15):
    return [types.SimpleNamespace(nant=nant, P=P, freqs=np.linspace(1e8, 2e8, 4),
                                  d_antpos=1, d_bm=2) for _ in range(n)]


def request(rid, nsrc, arrival=0.0, set_id=0, ntimes=2, nfreq=2):
    r = serve.Request(rid, set_id, nsrc, ntimes, nfreq, arrival)
    return serve.make_sky(r, seed=rid, lst0=0.1 * rid)


def run(reqs, budget=1e9, slots=2, max_batch=4):
    FakeBatch.launched = []
    ctxs = [FakeContext() for _ in range(slots)]
    srv = serve.Server(fake_sets(), ctxs, hbm_budget=budget, max_batch=max_batch,
                       batch_factory=FakeBatch)
    done = srv.run(reqs)
    for c in ctxs:
        assert not c.live, "device buffers leaked"
    return srv, done


def test_request_above_budget_is_rejected():
    sets = fake_sets()
    small = [request(i, 500) for i in range(6)]
    big = request(99, 2_000_000, ntimes=60, nfreq=16)
    budget = 4 * serve.request_bytes(small[0], sets[0].nant, sets[0].P)
    assert serve.request_bytes(big, sets[0].nant, sets[0].P) > budget
    srv, done = run(small + [big], budget=budget)
    assert big.error and "budget" in big.error and big.result is None
    assert all(r.ok for r in small)
    assert srv.max_held <= budget
    assert 2_000_000 not in FakeBatch.launched


def test_cancelled_request_is_never_launched():
    reqs = [request(i, 1000 + i, arrival=0.0) for i in range(5)]
    late = request(50, 4242, arrival=0.05)
    late.cancel()
    _, done = run(reqs + [late])
    assert late.error == "cancelled" and late.result is None
    assert 4242 not in FakeBatch.launched
    assert all(r.ok for r in reqs)
    stats = serve.summarize(done, 1.0)
    assert stats["cancelled"] == 1 and stats["served"] == 5


def test_failed_batches_fail_only_their_requests():
    good = [request(i, 1000 + i, arrival=0.001 * i) for i in range(8)]
    bad_launch = request(30, 13, arrival=0.02)
    bad_sync = request(31, 17, arrival=0.04)
    _, done = run(good + [bad_launch, bad_sync], max_batch=1)
    assert bad_launch.error.startswith("launch failed")
    assert bad_sync.error.startswith("batch failed")
    assert all(r.ok for r in good)
    stats = serve.summarize(done, 1.0)
    assert stats["failed"] == 2 and stats["served"] == 8


def test_budget_bounds_memory_in_flight():
    sets = fake_sets()
    reqs = [request(i, 3000, arrival=0.0) for i in range(12)]
    one = serve.request_bytes(reqs[0], sets[0].nant, sets[0].P)
    srv, _ = run(reqs, budget=2.5 * one, slots=4, max_batch=8)
    assert all(r.ok for r in reqs)
    assert one <= srv.max_held <= 2.5 * one


def test_results_handed_to_consumer_without_copy():
    reqs = [request(i, 800 + i, arrival=0.0) for i in range(6)]
    seen = {}

    def consume(r, view):
        seen[r.rid] = (view.shape, float(view.real.max()))

    FakeBatch.launched = []
    srv = serve.Server(fake_sets(), [FakeContext()], hbm_budget=1e9, max_batch=2,
                       batch_factory=FakeBatch)
    done = srv.run(reqs, on_result=consume)
    assert sorted(seen) == [r.rid for r in reqs]
    assert all(r.ok and r.delivered and r.result is None for r in done)
    assert all(shape == (r.nfreq, r.ntimes, 20, 20) and mx == 1.0
               for r in done for shape, mx in [seen[r.rid]])


def test_a_resident_set_that_fails_to_build_holds_no_device_memory():
    class FailingSecondAlloc(FakeContext):
        def device_alloc(self, nbytes):
            if self.live:
                raise _native.HeraVisError(_native.HV_ERR_OOM, "injected allocation failure")
            return super().device_alloc(nbytes)

    ctx = FailingSecondAlloc()
    with pytest.raises(_native.HeraVisError):
        serve.ResidentSet(ctx, np.zeros((4, 3)), [1e8], np.zeros((1, 4, 5, 5)))
    assert ctx.live == {}
    # a set that builds frees both buffers on close, once
    ctx = FakeContext()
    rs = serve.ResidentSet(ctx, np.zeros((4, 3)), [1e8], np.zeros((1, 4, 5, 5)))
    assert len(ctx.live) == 2
    rs.close()
    rs.close()
    assert ctx.live == {}


def test_batch_chunk_matches_the_library():
    # admission counts split-K partials with the library's chunk size
    src = open(os.path.join(os.path.dirname(serve.__file__), "csrc", "hv_batch.cu")).read()
    assert int(re.search(r"constexpr int kBatchChunk = (\d+);", src).group(1)) == serve.BATCH_CHUNK


def test_summary_splits_p99_by_arrival_half():
    # a queue that grows: the later arrivals wait longer
    reqs = []
    for i in range(100):
        r = request(i, 1000, arrival=0.01 * i)
        r.t_done = r.arrival + (0.01 if i < 50 else 0.5 + 0.01 * i)
        r.result = np.zeros(1)
        reqs.append(r)
    stats = serve.summarize(reqs, 2.0)
    assert stats["served"] == 100
    assert abs(stats["p99_first_half_ms"] - 10.0) < 1e-6
    assert stats["p99_second_half_ms"] > 1000.0
