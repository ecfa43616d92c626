"""Batched form: many uneven simulations planned and run together.

Each simulation of a batch must give what a single call gives for it (same
method, tensor cores), and the FP64 oracle within the tensor-core tolerance;
a batch replayed from its CUDA graph must give exactly the direct run.
"""
import numpy as np
import pytest

from hera_gpu_gb300 import _native, synth, vis_gpu_multifreq
from oracle import rel_frobenius, vis_oracle

pytestmark = pytest.mark.gpu

SIZES = [  # nant, nsrc, ntimes, nfreq, P   (cluster classes 1, 2 and 3 groups)
    (16, 1000, 3, 2, 31),
    (40, 3000, 2, 3, 31),
    (150, 2500, 2, 2, 63),
    (300, 4000, 1, 2, 63),
    (129, 700, 3, 1, 15),
    (350, 5000, 2, 2, 63),
    (20, 0, 2, 1, 7),      # no sources
]


def make(seed, nant, nsrc, ntimes, nfreq, P):
    cfg = synth.config_array(seed=seed, nant=nant, nsrc=nsrc, ntimes=ntimes, nfreq=nfreq,
                             fmin=100e6, fmax=200e6, P=P)
    bm = synth.beams_for(cfg, dtype=np.float32)
    return dict(antpos=cfg["antpos"].astype(np.float32), freqs=cfg["freqs"],
                eq2tops=cfg["eq2tops"].astype(np.float32),
                crd_eq=cfg["crd_eq"].astype(np.float32), I_sky=cfg["I_sky"].astype(np.float32),
                bm_cubes=bm)


@pytest.fixture(scope="module")
def batch_inputs():
    import torch
    dev = torch.device("cuda", 0)
    host, dev_arrays, sims = [], [], []
    for i, (nant, nsrc, nt, nf, P) in enumerate(SIZES):
        h = make(100 + i, nant, nsrc, nt, nf, P)
        d = {k: torch.from_numpy(np.ascontiguousarray(h[k])).to(dev)
             for k in ("antpos", "eq2tops", "crd_eq", "I_sky", "bm_cubes")}
        d["out"] = torch.full((nf, nt, nant, nant), float("nan"), dtype=torch.complex64, device=dev)
        host.append(h)
        dev_arrays.append(d)
        sims.append(dict(antpos=d["antpos"].data_ptr(), eq2tops=d["eq2tops"].data_ptr(),
                         crd_eq=d["crd_eq"].data_ptr(), I_sky=d["I_sky"].data_ptr(),
                         bm_cubes=d["bm_cubes"].data_ptr(), freqs=h["freqs"],
                         vis_out=d["out"].data_ptr(), nant=nant, ntimes=nt, nsrc=nsrc, beam_px=P))
    torch.cuda.synchronize()
    return host, dev_arrays, sims


def run(ctx, sims, dev_arrays, **kw):
    b = _native.Batch(ctx, sims, **kw)
    b.launch()
    b.sync()
    outs = [d["out"].cpu().numpy().copy() for d in dev_arrays]
    assert b.launches > 0
    b.close()
    return outs


def test_batch_matches_single_calls_and_oracle(batch_inputs):
    host, dev_arrays, sims = batch_inputs
    ctx = _native.Context(0)
    outs = run(ctx, sims, dev_arrays)
    for (nant, nsrc, nt, nf, P), h, o in zip(SIZES, host, outs):
        assert o.shape == (nf, nt, nant, nant)
        single = vis_gpu_multifreq(h["antpos"], h["freqs"], h["eq2tops"], h["crd_eq"], h["I_sky"],
                                   h["bm_cubes"], precision=1, method="tc", context=ctx)
        if nsrc == 0:
            np.testing.assert_equal(o, 0)
            continue
        assert rel_frobenius(o, single).max() <= 1e-5, (nant, nsrc)
        # the FP64 oracle on one frequency of the smaller simulations
        if nant * nsrc <= 150 * 3000:
            ref = vis_oracle(h["antpos"].astype(np.float64), h["freqs"][0],
                             h["eq2tops"].astype(np.float64), h["crd_eq"].astype(np.float64),
                             h["I_sky"].astype(np.float64), h["bm_cubes"][0].astype(np.float64))
            assert rel_frobenius(o[0], ref).max() <= 1e-4, (nant, nsrc)


def test_batch_graph_replay_is_exact(batch_inputs):
    host, dev_arrays, sims = batch_inputs
    ctx = _native.Context(0)
    direct = run(ctx, sims, dev_arrays)
    b = _native.Batch(ctx, sims, graph=True)
    for _ in range(2):
        for d in dev_arrays:
            d["out"].fill_(float("nan"))
        b.launch()
        b.sync()
        for d, ref in zip(dev_arrays, direct):
            np.testing.assert_array_equal(d["out"].cpu().numpy(), ref)
    b.close()


def test_batch_autotune(batch_inputs):
    host, dev_arrays, sims = batch_inputs
    ctx = _native.Context(0)
    direct = run(ctx, sims, dev_arrays)
    tuned = run(ctx, sims, dev_arrays, autotune=True)
    for (nant, nsrc, *_), a, b in zip(SIZES, direct, tuned):
        if nsrc:
            assert rel_frobenius(b, a).max() <= 1e-5
