"""Serving form: a continuous-batching request loop over the batched kernel.

The reference answers one ``vis_gpu`` call at a time (hera_gpu/vis.py:144);
a simulation service sees a stream of requests of uneven size.  This loop:

* keeps **resident sets** on the device -- an antenna layout and its beam
  cubes for a channel grid -- so a request only ships its sky (source
  directions and fluxes) and its LSTs;
* **admits** arrived requests into a batch when a slot (a context with its own
  stream) is free and the batch fits the HBM budget next to the batches in
  flight;
* runs each batch as one ``hv_batch`` (one persistent fused launch per
  cluster class over all of its requests), with the inputs copied in and the
  results copied out on the slot's stream, so batches on different slots
  overlap on the device while new requests keep arriving;
* records per request the latency from arrival to the result being in host
  memory, and reports p50 / p99 latency and the visibility throughput.

Failures stay with the requests they hit: a request that can never fit the
HBM budget is rejected on arrival, a cancelled request is dropped before it
is admitted, and a batch whose launch or device-side waits fail (a CUDA
error, a bounded wait that ran out) marks its own requests failed while the
loop goes on serving the others.

A request's result does not depend on which other requests share its batch:
every simulation of a batch keeps its own work items, split-K chunks and
reduction order.
"""
from __future__ import annotations

import collections
import time
from dataclasses import dataclass

import numpy as np

from . import _native, sky, synth


class ResidentSet:
    """An antenna layout and its beam cubes (nfreq, nant, P, P) on the device."""

    def __init__(self, ctx: _native.Context, antpos, freqs, bm_cubes):
        self.ctx = ctx
        antpos = np.ascontiguousarray(antpos, dtype=np.float32)
        bm = np.ascontiguousarray(bm_cubes, dtype=np.float32)
        self.nant = antpos.shape[0]
        self.P = bm.shape[-1]
        self.freqs = np.asarray(freqs, dtype=np.float64)
        self.nbytes = antpos.nbytes + bm.nbytes
        self.d_antpos = self.d_bm = 0
        try:
            self.d_antpos = ctx.device_alloc(antpos.nbytes)
            self.d_bm = ctx.device_alloc(bm.nbytes)
            ctx.h2d(self.d_antpos, antpos)
            ctx.h2d(self.d_bm, bm)
            ctx.sync()
        except Exception:
            self.close()    # a failed set holds no device memory
            raise

    def close(self):
        if self.d_antpos or self.d_bm:
            for ptr in (self.d_antpos, self.d_bm):
                if ptr:
                    self.ctx.device_free(ptr)
            self.ctx.sync()
            self.d_bm = self.d_antpos = 0


@dataclass
class Request:
    rid: int
    set_id: int
    nsrc: int
    ntimes: int
    nfreq: int
    arrival: float                  # seconds after the start of the run
    crd_eq: np.ndarray = None       # (3, nsrc) float32
    I_sky: np.ndarray = None        # (nsrc,) float32
    eq2tops: np.ndarray = None      # (ntimes, 3, 3) float32
    result: np.ndarray = None       # (nfreq, ntimes, nant, nant) complex64
    t_start: float = 0.0
    t_done: float = 0.0
    nant: int = 0
    error: str = None               # why the request was not served
    cancelled: bool = False
    delivered: bool = False         # result handed to the consumer callback

    def cancel(self):
        """Drop the request if it has not been admitted yet."""
        self.cancelled = True

    @property
    def ok(self):
        return self.error is None and (self.result is not None or self.delivered)

    @property
    def latency(self):
        return self.t_done - self.arrival

    @property
    def visibilities(self):
        return self.nfreq * self.ntimes * self.nant * self.nant


def make_sky(req: Request, seed: int, lst0: float):
    """Seeded sky and LSTs of a request (sphere-uniform power-law sources)."""
    rng = np.random.default_rng(seed)
    req.crd_eq = synth.sphere_sources(req.nsrc, rng).astype(np.float32)
    req.I_sky = synth.powerlaw_flux(req.nsrc, -2.0, 0.05, 50.0, rng).astype(np.float32)
    lsts = sky.lst_grid(req.ntimes, 1.0, start_rad=lst0)
    req.eq2tops = sky.eq2tops(lsts, np.radians(sky.HERA_LATITUDE_DEG)).astype(np.float32)
    return req


# sources per split-K chunk of a simulation in a batch (hv_batch.cu)
BATCH_CHUNK = 65536


def request_bytes(req: Request, nant: int, P: int) -> int:
    """Device memory one request holds while in flight (inputs, output and its
    share of the batch workspace), for admission against the HBM budget.  The
    loop's batches are not autotuned, so a slice has ceil(nsrc / BATCH_CHUNK)
    split-K chunks (an autotuned divisor would multiply them)."""
    Np = -(-nant // 128) * 128
    T, F, S = req.ntimes, req.nfreq, max(req.nsrc, 1)
    nchunk = -(-S // BATCH_CHUNK)  # split-K chunks per slice of the batched kernel
    inputs = 16 * S + 36 * T
    out = 8 * F * T * nant * nant
    work = (4 * F * P * P * Np + 32 * T * F * Np + 32 * T * (S + 32) + 24 * S
            + 8 * T * F * nchunk * Np * Np + 8 * 2 ** int(np.ceil(np.log2(max(S, 2048)))))
    return inputs + out + work


@dataclass
class _InFlight:
    slot: int
    batch: object
    reqs: list
    buffers: list
    outs: list
    nbytes: int


class _PinnedRing:
    """Page-locked staging of one slot: request inputs and results of the
    batch in flight on that slot.  It is reallocated (doubled) only while the
    slot is idle, and rarely: freeing page-locked memory waits for the whole
    device, other slots included."""

    def __init__(self, ctx, nbytes=64 << 20):
        self.ctx = ctx
        self.buf = ctx.pinned_empty((nbytes,), np.uint8)
        self.off = 0

    def reset(self, need):
        if need > self.buf.nbytes:
            size = self.buf.nbytes
            while size < need:
                size *= 2
            self.buf = None
            self.buf = self.ctx.pinned_empty((size,), np.uint8)
        self.off = 0

    def take(self, shape, dtype):
        dtype = np.dtype(dtype)
        n = int(np.prod(shape)) * dtype.itemsize
        a = self.buf[self.off:self.off + n].view(dtype).reshape(shape)
        self.off += (n + 255) // 256 * 256
        return a


class Server:
    """Continuous-batching loop over ``slots`` device streams (one context
    each).  ``batch_factory(ctx, sims)`` builds a batch (default
    :class:`_native.Batch`)."""

    def __init__(self, sets, contexts, hbm_budget=150e9, max_batch=64, batch_factory=None):
        self.sets = sets
        self.ctxs = contexts
        self.budget = float(hbm_budget)
        self.max_batch = int(max_batch)
        self.batch_factory = batch_factory or _native.Batch
        self.rings = [_PinnedRing(c) for c in contexts]
        self.max_held = 0.0  # largest device memory admitted at once (bytes)

    def _staging_bytes(self, r):
        rs = self.sets[r.set_id]
        return (sum(getattr(r, n).nbytes + 256 for n in ("crd_eq", "I_sky", "eq2tops"))
                + 8 * r.nfreq * r.ntimes * rs.nant * rs.nant + 256)

    def reserve(self, requests, cap_bytes=2 << 30):
        """Size every slot's page-locked staging for the ``max_batch``
        largest of ``requests`` (at most ``cap_bytes``), so that serving
        them allocates no page-locked memory."""
        sizes = sorted((self._staging_bytes(r) for r in requests), reverse=True)
        need = min(sum(sizes[:self.max_batch]), cap_bytes)
        for ring in self.rings:
            ring.reset(need)

    def _launch(self, slot, reqs):
        """Copy the requests' inputs in, launch their batch and queue the
        result copies, all on the slot's stream.  Returns the in-flight record,
        or None when the launch failed (the requests then carry the error)."""
        ctx = self.ctxs[slot]
        ring = self.rings[slot]
        ring.reset(sum(self._staging_bytes(r) for r in reqs))
        bufs, outs, sims = [], [], []
        nbytes = sum(request_bytes(r, self.sets[r.set_id].nant, self.sets[r.set_id].P)
                     for r in reqs)
        batch = None
        try:
            for r in reqs:
                rs = self.sets[r.set_id]
                r.nant = rs.nant
                d = {}
                for name in ("crd_eq", "I_sky", "eq2tops"):
                    a = getattr(r, name)
                    h = ring.take(a.shape, a.dtype)
                    h[...] = a
                    d[name] = ctx.device_alloc(a.nbytes)
                    bufs.append(d[name])
                    ctx.h2d(d[name], h)
                out = ring.take((r.nfreq, r.ntimes, rs.nant, rs.nant), np.complex64)
                outs.append(out)
                d["out"] = ctx.device_alloc(out.nbytes)
                bufs.append(d["out"])
                sims.append(dict(antpos=rs.d_antpos, eq2tops=d["eq2tops"], crd_eq=d["crd_eq"],
                                 I_sky=d["I_sky"], bm_cubes=rs.d_bm, freqs=rs.freqs[:r.nfreq],
                                 vis_out=d["out"], nant=rs.nant, ntimes=r.ntimes, nsrc=r.nsrc,
                                 beam_px=rs.P))
            batch = self.batch_factory(ctx, sims)
            batch.launch()
        except _native.HeraVisError as e:
            if batch is not None:
                batch.close()
            for b in bufs:
                ctx.device_free(b)
            for r in reqs:
                r.error = f"launch failed: {e}"
            return None
        for out, s in zip(outs, sims):
            ctx.d2h(out, s["vis_out"])
        return _InFlight(slot, batch, reqs, bufs, outs, nbytes)

    def run(self, requests, clock=time.perf_counter, poll_s=2e-4, on_result=None):
        """Serve ``requests`` (sorted by arrival, seconds from now); returns
        them with timings.  Each result lands in the slot's page-locked
        staging; by default it is copied into ``request.result``.  With
        ``on_result(request, view)`` the consumer gets the staged result
        itself instead (no host copy) and must copy what it keeps before
        returning: the slot reuses the staging for its next batch."""
        requests = sorted(requests, key=lambda r: r.arrival)
        pending = collections.deque()
        inflight = {}
        held = 0.0
        i = 0
        t0 = clock()
        while i < len(requests) or pending or inflight:
            now = clock() - t0
            while i < len(requests) and requests[i].arrival <= now:
                pending.append(requests[i])
                i += 1
            progressed = False
            for slot in list(inflight):
                f = inflight[slot]
                if self.ctxs[slot].idle():
                    try:
                        f.batch.sync()  # device-side errors of the batch (timeouts)
                        err = None
                    except _native.HeraVisError as e:
                        err = f"batch failed: {e}"
                    t = clock() - t0  # the results are in host memory
                    for r, out in zip(f.reqs, f.outs):
                        r.t_done = t
                        if err is not None:
                            r.error = err
                        elif on_result is None:
                            r.result = out.copy()
                        else:
                            on_result(r, out)
                            r.delivered = True
                    f.batch.close()
                    for b in f.buffers:
                        self.ctxs[slot].device_free(b)
                    held -= f.nbytes
                    del inflight[slot]
                    progressed = True
            for slot in range(len(self.ctxs)):
                if slot in inflight or not pending:
                    continue
                take, nb = [], 0.0
                while pending and len(take) < self.max_batch:
                    r = pending[0]
                    rs = self.sets[r.set_id]
                    need = request_bytes(r, rs.nant, rs.P)
                    if r.cancelled or need > self.budget:
                        # never admitted: cancelled, or larger than the budget
                        pending.popleft()
                        r.error = "cancelled" if r.cancelled else (
                            f"needs {need / 1e9:.2f} GB, above the HBM budget of "
                            f"{self.budget / 1e9:.2f} GB")
                        r.t_done = clock() - t0
                        progressed = True
                        continue
                    if held + nb + need > self.budget:
                        break  # wait for memory to free up
                    take.append(pending.popleft())
                    nb += need
                if not take:
                    continue
                t = clock() - t0
                for r in take:
                    r.t_start = t
                f = self._launch(slot, take)
                progressed = True
                if f is None:  # the launch failed: its requests carry the error
                    for r in take:
                        r.t_done = clock() - t0
                    continue
                inflight[slot] = f
                held += f.nbytes
                self.max_held = max(self.max_held, held)
            if not progressed:
                nxt = requests[i].arrival - (clock() - t0) if i < len(requests) else poll_s
                time.sleep(max(0.0, min(poll_s, nxt)))
        return requests


def summarize(requests, wall_s):
    """Latency percentiles and throughput over the served requests."""
    done = [r for r in requests if r.ok]
    lat = np.array([r.latency for r in done]) if done else np.zeros(1)
    vis = sum(r.visibilities for r in done)
    # steady state: the p99 of the requests that arrived in the first and in
    # the second half of the run (a loop that keeps up shows no growth)
    by_arrival = sorted(done, key=lambda r: r.arrival)
    half = len(by_arrival) // 2

    def p99(rs):
        return float(np.percentile([r.latency for r in rs], 99) * 1e3) if rs else 0.0

    return {"requests": len(requests), "served": len(done),
            "failed": sum(1 for r in requests if r.error and not r.cancelled),
            "cancelled": sum(1 for r in requests if r.cancelled),
            "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "p99_first_half_ms": p99(by_arrival[:half]),
            "p99_second_half_ms": p99(by_arrival[half:]),
            "mean_ms": float(lat.mean() * 1e3), "vis_per_s": vis / wall_s, "wall_s": wall_s}


def workload(nreq, rate_hz=200.0, large_frac=0.05, nsets=8, seed=0, large=(350, 1_048_576, 60),
             max_nsrc=200_000):
    """Request stream of the serving configuration: Poisson arrivals at
    ``rate_hz``; sizes from the batched-form distribution (nsrc log-uniform in
    [1e3, 2e5], ntimes in [1, 60], nfreq in [1, 16]) on ``nsets`` resident
    sets, plus ``large_frac`` large requests (nant 350, 1M sources, 60 LSTs;
    they use a 350-antenna set).  Returns (set specs, requests) -- set specs
    are dicts for :func:`build_sets`."""
    rng = np.random.default_rng(seed)
    specs = []
    for k in range(nsets):
        nant = 350 if k == 0 else int(np.round(np.exp(rng.uniform(np.log(16), np.log(350)))))
        specs.append(dict(seed=int(rng.integers(1 << 30)), nant=nant,
                          P=int(rng.choice([31, 63]))))
    t = 0.0
    reqs = []
    for rid in range(nreq):
        t += rng.exponential(1.0 / rate_hz)
        if rng.random() < large_frac:
            set_id, nsrc, ntimes, nfreq = 0, large[1], large[2], 1
        else:
            set_id = int(rng.integers(nsets))
            nsrc = int(np.round(np.exp(rng.uniform(np.log(1e3), np.log(max_nsrc)))))
            ntimes = int(rng.integers(1, 61))
            nfreq = int(rng.integers(1, 17))
        req = Request(rid, set_id, nsrc, ntimes, nfreq, t)
        make_sky(req, seed=int(rng.integers(1 << 30)), lst0=float(rng.uniform(0, 2 * np.pi)))
        reqs.append(req)
    return specs, reqs


def build_sets(ctx, specs, nfreq=16):
    """Resident sets: hex-subset layouts with Airy beams on ``nfreq`` channels
    over 100-200 MHz."""
    sets = []
    for sp in specs:
        rng = np.random.default_rng(sp["seed"])
        full = synth.hex_array(350, 14.6, 0.01, rng)
        pick = np.sort(rng.choice(350, size=sp["nant"], replace=False))
        dish = 14.0 * (1.0 + 0.02 * rng.uniform(-1.0, 1.0, sp["nant"]))
        freqs = np.linspace(100e6, 200e6, nfreq)
        bm = np.stack([synth.airy_beams(sp["nant"], sp["P"], f, dish) for f in freqs]).astype(np.float32)
        sets.append(ResidentSet(ctx, full[pick], freqs, bm))
    return sets
