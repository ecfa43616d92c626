"""Throughput of the visibility simulator on GB300 (one JSON line on rank 0).

Workload (the precision-form configuration): 350 antennas on a 14.6 m hex
grid, 1,048,576 sphere-uniform power-law sources, 64 channels evenly spaced
on 100-200 MHz with per-channel 350x63x63 Airy beam cubes, LSTs over one
hour at latitude -30.72 deg; seeded synthetic data.  One step = one call of
the hot path over 4 consecutive LSTs (of 120) and all 64 channels, i.e.
4 * 64 * 350**2 visibilities.

Arms
  (default)          fused tensor-core form through the C ABI, inputs resident
                     in HBM (``value``); the same call through the public
                     Python API with page-locked host buffers, copies inside
                     the timed region (``e2e``); the plain FP32 form on one
                     step for comparison; the CPU oracle port on a bounded
                     sample (``cpu_baseline``).
  --impl reference   the reference's CPU algorithm (the oracle port of
                     hera_gpu/tests/test_vis_gpu.py:278-357) on the host
                     cores, on a bounded sample of the same workload.

Also timed: the plain FP32 form on the same step, the array-scale and
small configurations (350 x 100k x 60 LSTs in FP32, tensor-core and FP64;
16 x 1000 x 10 LSTs), and each output's error against the FP64 oracle on
whole (time, channel) slices at the corners of the configuration (first and
last LST x lowest and highest channel).

Several GPUs run independent replicas (the path has no exchange step):
``--gpus N`` without a torchrun environment launches N ranks itself through
torch.distributed.run, one replica per GPU, and the job's time is the
slowest rank's.
"""
from __future__ import annotations

import argparse
import contextlib
import json
import math
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NANT, NSRC, NFREQ, NTIMES, BEAM_PX = 350, 1_048_576, 64, 120, 63
T_PER_STEP = 4
FMIN, FMAX = 100e6, 200e6
CPU_SAMPLE_SRC = 16384          # sources per host process per CPU sample
CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nsrc", type=int, default=NSRC)
    ap.add_argument("--nfreq", type=int, default=NFREQ)
    ap.add_argument("--nant", type=int, default=NANT)
    ap.add_argument("--method", default="tc", choices=["tc", "tc_fp16", "plain"])
    ap.add_argument("--no-forms", action="store_true",
                    help="skip timing the other fused form on the same steps")
    ap.add_argument("--stages", type=int, default=0,
                    help="fused kernel: cap on operand stages in shared memory (0 = default)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-form comparison")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=2000,
                    help="requests of the serving leg (0 = skip); at 200 req/s, 2000 requests "
                         "arrive over about 10 s, long enough to compare the p99 of the two "
                         "halves of the run")
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-rate-low", type=float, default=100.0,
                    help="a second serving run at this rate (0 = skip)")
    ap.add_argument("--serve-slots", type=int, default=4)
    ap.add_argument("--serve-max-batch", type=int, default=2)
    ap.add_argument("--batch-sims", type=int, default=256,
                    help="simulations of the batched-form leg (0 = skip)")
    ap.add_argument("--no-median", action="store_true", help="skip the median-filter leg")
    ap.add_argument("--median-only", action="store_true",
                    help="run only the median-filter leg and print its summary")
    ap.add_argument("--no-omnical", action="store_true", help="skip the omnical leg")
    ap.add_argument("--omnical-only", action="store_true",
                    help="run only the omnical leg and print its summary")
    ap.add_argument("--omnical-cases", default="",
                    help="omnical cases as nants:precision,... (default: the reference's four)")
    ap.add_argument("--batch-only", action="store_true",
                    help="run only the batched-form leg and print its summary")
    ap.add_argument("--serve-only", action="store_true",
                    help="run only the serving leg and print its summary (profiling runs)")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the array-scale and small-configuration legs")
    ap.add_argument("--no-corners", action="store_true",
                    help="skip the per-(time, channel) error check at the configuration's corners")
    ap.add_argument("--dry-run", action="store_true",
                    help="launcher check without a GPU: every rank times an empty step over a "
                         "gloo process group and rank 0 prints the line")
    return ap.parse_args()


# ----------------------------------------------------------------- workload --
def make_workload(nant, nsrc, nfreq, seed=0):
    import numpy as np
    from hera_gpu_gb300 import synth
    cfg = synth.config_array(seed=seed, nant=nant, nsrc=nsrc, ntimes=NTIMES, nfreq=nfreq,
                             fmin=FMIN, fmax=FMAX, P=BEAM_PX)
    w = dict(antpos=cfg["antpos"].astype(np.float32), freqs=cfg["freqs"],
             eq2tops=cfg["eq2tops"].astype(np.float32), crd_eq=cfg["crd_eq"].astype(np.float32),
             I_sky=cfg["I_sky"].astype(np.float32))
    w["bm_cubes"] = synth.beams_for(cfg, dtype=np.float32)
    return w


def sources_up(w, t):
    """Sources above the horizon at time t (FP64, as the prep kernel)."""
    import numpy as np
    z = np.asarray(w["eq2tops"][t], dtype=np.float64)[2] @ np.asarray(w["crd_eq"], dtype=np.float64)
    return int(np.count_nonzero(z > 0))


def tc_chunk(nsrc, nslices, ngroups, num_sms):
    """Split-K chunk the library picks (hv_tc.cu tc_chunk_sources)."""
    nchunk = max(1, -(-40 * num_sms // (nslices * ngroups)))
    c = -(-max(nsrc // 2, 1) // nchunk)
    c = min(16384, max(1024, c))
    return (c + 31) // 32 * 32


def tc_groups(nant):
    """The fused kernel's block-pair groups (hv_tc.cu make_groups): per group
    its MMA N.  Pairs (I, J), (I, J + 1) share row block I; the pairs left
    over at the end of a row, (I, nb - 1), are taken as (nb - 1, I) and
    paired in ascending I."""
    nb = (nant + 127) // 128
    ncols = [(min(128, nant - 128 * b) + 15) // 16 * 16 for b in range(nb)]
    groups, singles = [], []
    for I in range(nb):
        J = I
        while J + 1 < nb:
            groups.append(128 + ncols[J + 1])
            J += 2
        if J < nb:
            singles.append(I)
    for k in range(0, len(singles), 2):
        groups.append(128 + ncols[singles[k + 1]] if k + 1 < len(singles) else ncols[singles[k]])
    return groups


def tc_num_groups(nant):
    return len(tc_groups(nant))


# ------------------------------------------------------------------- clocks --
class ClockSampler:
    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={CLOCK_FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            lines = open(self.path).read().strip().splitlines()
        except OSError:
            lines = []
        for ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if self.path:
            os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# -------------------------------------------------------------- CPU oracle --
def _cpu_worker(args):
    """One host process: the oracle port on one block of sources (checker and
    CPU baseline only)."""
    import numpy as np
    from oracle import vis_oracle_partial
    antpos, freq, eq2top, crd, I, bm, dt = args
    t0 = time.perf_counter()
    V = vis_oracle_partial(antpos, freq, eq2top, crd, I, bm.astype(dt), 0, crd.shape[1], dtype=dt)
    return V, time.perf_counter() - t0


def cpu_pool():
    """One single-threaded oracle process per host core (spawned, so it is
    safe before or after CUDA initialisation)."""
    import multiprocessing as mp
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    for k in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[k] = "1"
    return mp.get_context("spawn").Pool(cores), cores


def cpu_sample(pool, cores, w, t, f, dtype="float64", nsamp=None):
    """Oracle on nsamp (default cores x CPU_SAMPLE_SRC) sources of slice
    (t, f), one block of sources per process, in float64 (the FP64 oracle) or float32 (the
    arithmetic of the reference's precision-1 CPU path); returns (V of the
    sample, seconds, sources).  The seconds are the longest per-process
    compute time (the parallel span, without the inter-process transfer of
    inputs)."""
    import numpy as np
    nsamp = min(nsamp or cores * CPU_SAMPLE_SRC, w["crd_eq"].shape[1])
    bounds = np.linspace(0, nsamp, cores + 1).astype(int)
    a64 = lambda x: np.asarray(x, dtype=np.float64)
    jobs = [(a64(w["antpos"]), float(w["freqs"][f]), a64(w["eq2tops"][t]),
             a64(w["crd_eq"][:, bounds[i]:bounds[i + 1]]), a64(w["I_sky"][bounds[i]:bounds[i + 1]]),
             np.asarray(w["bm_cubes"][f]), np.dtype(dtype)) for i in range(cores)]
    parts = pool.map(_cpu_worker, jobs)
    span = max(p[1] for p in parts)
    return sum(p[0] for p in parts), span, nsamp


def cpu_rate(wall, nsamp, nant, nsrc_full):
    """vis/s of the CPU path on a full slice, extrapolated linearly in sources."""
    t_slice = wall * nsrc_full / nsamp
    return nant * nant / t_slice


# ------------------------------------------------------------------ ranks --
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x, device=None):
    """The largest of every rank's x (the job's time is its slowest
    replica's); x itself without a process group."""
    import torch
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, world, seconds):
    """Whole-job throughput of `world` replicas that each processed
    units_per_rank units in (at most) `seconds`."""
    return world * units_per_rank / seconds


def step_config(args, world):
    """The workload of one step: the same dict in both arms."""
    return {"workload": f"{args.nant} ant x {args.nsrc} src x {args.nfreq} ch (100-200 MHz), "
                        f"{T_PER_STEP} of {NTIMES} LSTs per step, beams {BEAM_PX}x{BEAM_PX}",
            "nant": args.nant, "nsrc": args.nsrc, "nfreq": args.nfreq,
            "ntimes_per_step": T_PER_STEP, "l2": "inputs larger than L2",
            "parallelism": f"replicas x{world}"}


def run_reference(args):
    """The reference's CPU algorithm (the oracle port of vis_cpu) on the host
    cores.  Each step is a bounded sample of the workload: every host process
    takes a block of CPU_SAMPLE_SRC sources of one (time, channel) slice, in
    float32 (the reference's default precision=1, hera_gpu/vis.py:146); the
    rate is extrapolated linearly to the slice's full source count.  One
    float64 sample (precision=2) is reported beside it."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    import numpy as np
    pool, cores = cpu_pool()
    w = make_workload(args.nant, args.nsrc, args.nfreq)
    rates, walls = [], []
    for i in range(args.warmup + args.steps):
        t = (i * T_PER_STEP) % NTIMES
        t0 = time.perf_counter()
        _, span, nsamp = cpu_sample(pool, cores, w, t, i % args.nfreq, "float32")
        if i >= args.warmup:
            walls.append(time.perf_counter() - t0)
            rates.append(cpu_rate(span, nsamp, args.nant, args.nsrc))
    _, span64, nsamp64 = cpu_sample(pool, cores, w, 0, 0, "float64")
    pool.close()
    value = float(np.mean(rates))
    sample = (f"{cores} host processes x {CPU_SAMPLE_SRC} sources of one (time, channel) slice "
              f"per step in float32 (the reference's default precision 1), extrapolated "
              f"linearly to {args.nsrc} sources; ms_per_step is the sample's wall time")
    line = {
        "impl": "reference", "metric": "visibilities/s", "value": value, "unit": "vis/s",
        "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * float(np.mean(walls)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)", "method": "cpu",
        "config": step_config(args, world),
        "cpu_baseline": {"value": value, "unit": "vis/s", "cores": cores, "kind": "port",
                         "sample": sample,
                         "value_fp64": cpu_rate(span64, nsamp64, args.nant, args.nsrc)},
        "e2e": {"value": value, "unit": "vis/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def launch_replicas(args):
    """``--gpus N`` outside a torchrun environment: run this script as N
    ranks through torch.distributed.run (one replica per GPU, rendezvous on
    127.0.0.1) and return its exit status; None when this process is already
    a rank (or N is 1)."""
    if args.gpus <= 1 or "WORLD_SIZE" in os.environ:
        return None
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           f"--nproc-per-node={args.gpus}", "--master-addr", "127.0.0.1",
           "--master-port", str(port), os.path.abspath(__file__), *sys.argv[1:]]
    return subprocess.call(cmd)


def run_dry(args):
    """The replica launcher and the max-over-ranks timing without a GPU:
    each rank times an empty step; rank 0 prints a line with n_gpus = the
    number of ranks."""
    import torch
    import torch.distributed as dist
    world, rank, _ = dist_setup()
    if world > 1:
        dist.init_process_group("gloo")
    t0 = time.perf_counter()
    time.sleep(0.01 * (rank + 1))
    ms = max_over_ranks(1e3 * (time.perf_counter() - t0))
    if rank == 0:
        print(json.dumps({"metric": "visibilities/s", "dry_run": True, "n_gpus": world,
                          "ms_per_step": ms, "config": step_config(args, world)}), flush=True)
    if world > 1:
        dist.destroy_process_group()
    del torch
    return 0


def load_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


# DRAM bytes per unit of work (slice x source above the horizon) of one
# fused-kernel launch, measured once with ncu (dram__bytes_read.sum +
# dram__bytes_write.sum of the launch on 350 antennas x 1,048,576 sources x
# 16 channels x 4 LSTs, which under ncu computes all 33,517,808 units:
# split BF16 2.367 GB, FP16 + FP8 2.615 GB): the bench cannot read DRAM
# counters itself, so the figure is carried here and scaled by the units
# each timed launch processed.  That launch uses split-K chunks of 16384
# sources; the 64-channel benchmark call uses chunks of 32768, with half
# as many partial sums to write, so for it the figure is an upper bound
# (a full-size capture of these counters takes several ncu passes, more
# than a capture of that size may).
TC_DRAM_BYTES_PER_UNIT = {"tc": 70.619, "tc_fp16": 78.013}


def run_leg(fn, *a):
    """One leg of the line after the headline: its result, or its failure (a
    library error, a device-side wait that gave up) reported in its own
    object instead of taking the whole line down (the traceback goes to
    stderr)."""
    try:
        return fn(*a)
    except Exception as e:  # noqa: BLE001 -- reported in the JSON line
        import traceback
        traceback.print_exc()
        return {"error": f"{type(e).__name__}: {e}"}


def run_ours(args):
    import numpy as np
    world, rank, local = dist_setup()
    pool = cores = None
    if rank == 0 and not args.no_cpu:
        pool, cores = cpu_pool()      # spawned before the first CUDA call
    import torch
    from hera_gpu_gb300 import _native, vis_gpu_multifreq
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    ctx = _native.Context(local)
    ctx.set_tuning(stages=args.stages)
    num_sms = torch.cuda.get_device_properties(local).multi_processor_count
    w = make_workload(args.nant, args.nsrc, args.nfreq, seed=rank)
    N, S, F = args.nant, args.nsrc, args.nfreq
    dev = torch.device("cuda", local)
    d = {k: torch.from_numpy(np.ascontiguousarray(w[k])).to(dev)
         for k in ("antpos", "eq2tops", "crd_eq", "I_sky", "bm_cubes")}
    d_out = torch.empty((F, T_PER_STEP, N, N), dtype=torch.complex64, device=dev)
    torch.cuda.synchronize(dev)
    # a stream of our own: the library launches on it and the events time it
    stream = torch.cuda.Stream(dev)

    def step(i, method, t0=None):
        t0 = (i * T_PER_STEP) % NTIMES if t0 is None else t0
        ctx.vis_multifreq_device(1, method, d["antpos"].data_ptr(), N, w["freqs"],
                                 d["eq2tops"][t0:t0 + T_PER_STEP].data_ptr(), T_PER_STEP,
                                 d["crd_eq"].data_ptr(), d["I_sky"].data_ptr(), S,
                                 d["bm_cubes"].data_ptr(), BEAM_PX, d_out.data_ptr(),
                                 stream.cuda_stream)
        return t0

    def barrier():
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()

    # ---- device-resident throughput of a form --------------------------------
    vis_per_step = T_PER_STEP * F * N * N
    peaks, peak_src = load_peaks()

    def time_form(method, sample_clocks):
        for i in range(args.warmup):
            step(i, method)
        ctx.sync()
        barrier()
        ctx.set_profiling(True)
        ctx.profile_read()
        l0 = ctx.launches
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        times = []
        sampler = ClockSampler(local) if sample_clocks else contextlib.nullcontext()
        with sampler as clocks:
            barrier()
            ev0.record(stream)
            for i in range(args.warmup, args.warmup + args.steps):
                times.append(step(i, method))
            ev1.record(stream)
            barrier()
        ms = ev0.elapsed_time(ev1)
        ctx.sync()
        kern_ms, kern_launches = ctx.profile_read()
        ctx.set_profiling(False)
        return dict(ms=max_over_ranks(ms, dev), kern_ms=kern_ms, kern_launches=kern_launches,
                    launches=ctx.launches - l0, times=times,
                    clocks=clocks.summary() if sample_clocks else None)

    def roofline(method, r):
        """Roofline of the contraction kernel of one timed form."""
        s_up = [sources_up(w, t0 + k) for t0 in r["times"] for k in range(T_PER_STEP)]
        herk_flops = sum(4.0 * N * (N + 1) * su * F for su in s_up)
        kern_s = r["kern_ms"] / 1e3
        if method in ("tc", "tc_fp16"):
            ks, mmas = (16, 12) if method == "tc" else (32, 16)
            chunk = tc_chunk(S, T_PER_STEP * F, tc_num_groups(N), num_sms)
            stages = sum(sum(math.ceil(min(chunk, su - k0) / ks) for k0 in range(0, su, chunk))
                         for su in s_up) * F
            # tensor-pipe work in units of an M128 K16 BF16 MMA (an FP8 MMA
            # of K = 32 takes the same time)
            hw_flops = stages * mmas * 2 * 128 * 16 * sum(tc_groups(N))
            peak = peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops"))
            traffic_unit = TC_DRAM_BYTES_PER_UNIT.get(method)
            units = sum(s_up) * F
            return {"bound": "tensor", "achieved": herk_flops / kern_s / 1e12,
                    "peak": peak, "unit": "TFLOP/s", "frac": herk_flops / kern_s / 1e12 / peak,
                    "traffic": (traffic_unit * units / r["kern_launches"]) if traffic_unit else None,
                    "kernel": "tc_vis_kernel", "launches": r["kern_launches"],
                    "kernel_ms": r["kern_ms"],
                    "hw_tflops": hw_flops / kern_s / 1e12,
                    "hw_frac": hw_flops / kern_s / 1e12 / peak,
                    "peak_kind": f"bf16 dense sustained ({peak_src})",
                    "algorithmic": "4 N (N+1) S_up flops per slice (Hermitian upper triangle); "
                                   "hw_* counts the issued MMAs in BF16 M128 K16 equivalents "
                                   + ("(3 split-BF16 products, 128-blocks)" if method == "tc" else
                                      "(FP16 hi product + 2 FP8 cross products, 128-blocks)")}
        peak = 152 * 128 * 2 * 1.92e9 / 1e12
        return {"bound": "fp32-simt", "achieved": herk_flops / kern_s / 1e12, "peak": peak,
                "unit": "TFLOP/s", "frac": herk_flops / kern_s / 1e12 / peak, "traffic": None,
                "kernel": "herk_plain_kernel", "launches": r["kern_launches"],
                "kernel_ms": r["kern_ms"]}

    head = time_form(args.method, True)
    ms = head["ms"]
    value = job_rate(args.steps * vis_per_step, world, ms / 1e3)
    clk = head["clocks"]
    launches = head["launches"]
    roof = roofline(args.method, head)
    # the other fused form on the same steps
    other = {"tc": "tc_fp16", "tc_fp16": "tc"}.get(args.method)
    forms = {}
    if other and not args.no_forms:
        r = time_form(other, False)
        forms[other] = {"value": job_rate(args.steps * vis_per_step, world, r["ms"] / 1e3),
                        "ms_per_step": r["ms"] / args.steps, "gpu_launches": r["launches"],
                        "roofline": roofline(other, r)}

    line = {
        "metric": "visibilities/s", "value": value, "unit": "vis/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"tc": "bf16", "tc_fp16": "fp16+e4m3"}.get(args.method, "fp32"),
        "data": "synthetic (seeded); inputs larger than L2 (beam cubes "
                f"{w['bm_cubes'].nbytes / 1e6:.0f} MB)",
        "method": args.method, "config": step_config(args, world),
        "roofline": roof, "clocks": clk, "gpu_launches": launches, "forms": forms,
        # the reference returns the full N x N matrix (the metric above); the
        # distinct baselines a b >= a of it are N (N + 1) / 2 of those
        "unique_baselines_per_s": value * (N + 1) / (2.0 * N),
    }

    # ---- end to end through the public API, host buffers -----------------
    if not args.no_e2e:
        pin = {k: ctx.pinned_empty(w[k].shape, w[k].dtype) for k in
               ("antpos", "crd_eq", "I_sky", "bm_cubes")}
        for k in pin:
            pin[k][...] = w[k]
        e2t = ctx.pinned_empty((T_PER_STEP, 3, 3), np.float32)
        out = ctx.pinned_empty((F, T_PER_STEP, N, N), np.complex64)

        def e2e_step(i):
            t0 = (i * T_PER_STEP) % NTIMES
            e2t[...] = w["eq2tops"][t0:t0 + T_PER_STEP]
            vis_gpu_multifreq(pin["antpos"], w["freqs"], e2t, pin["crd_eq"], pin["I_sky"],
                              pin["bm_cubes"], precision=1, method=args.method, context=ctx,
                              out=out)
            return float(out[0, 0, 0, 0].real)   # read of the step's result
        e2e_step(0)
        barrier()
        t0 = time.perf_counter()
        for i in range(args.steps):
            e2e_step(i)
        e2e_s = max_over_ranks(time.perf_counter() - t0, dev)
        h2d = sum(pin[k].nbytes for k in pin) + e2t.nbytes + 8 * F
        line["e2e"] = {"value": job_rate(args.steps * vis_per_step, world, e2e_s), "unit": "vis/s",
                       "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(out.nbytes),
                       "api": "hera_gpu_gb300.vis_gpu_multifreq -> hv_vis_multifreq"}

    # ---- the plain FP32 form on one step (the method of the reference) ----
    if rank == 0 and not args.no_plain and args.method != "plain":
        step(0, "plain")
        ctx.sync()
        ctx.set_profiling(True)
        ctx.profile_read()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step(1, "plain")
        e1.record(stream)
        torch.cuda.synchronize(dev)
        pms = e0.elapsed_time(e1)
        pk_ms, _ = ctx.profile_read()
        ctx.set_profiling(False)
        pflops = sum(4.0 * N * (N + 1) * sources_up(w, T_PER_STEP + k) * F
                     for k in range(T_PER_STEP))
        line["plain_fp32"] = {"value": vis_per_step / (pms / 1e3), "unit": "vis/s",
                              "ms_per_step": pms,
                              "herk_tflops": pflops / (pk_ms / 1e3) / 1e12,
                              "tc_speedup": value / world / (vis_per_step / (pms / 1e3))}

    # ---- error against the FP64 oracle at the corners of the configuration
    # (first and last LST x lowest and highest channel), whole slices with
    # all S sources, each form's output from a call of the timed shape (4
    # LSTs x all channels, the benchmark's own split-K chunking) -------------
    if rank == 0 and pool is not None:
        methods = [args.method] + list(forms) + (["plain"] if not args.no_plain and
                                                 args.method != "plain" else [])
        corners = [(0, 0), (0, F - 1), (NTIMES - 1, 0), (NTIMES - 1, F - 1)]
        if args.no_corners:
            corners = corners[:1]
        got = {m: {} for m in methods}
        for m in methods:
            for t0 in sorted({min(t, NTIMES - T_PER_STEP) for t, _ in corners}):
                step(0, m, t0)
                torch.cuda.synchronize(dev)   # the call ran on `stream`
                ctx.sync()
                for t, f in corners:
                    if t0 <= t < t0 + T_PER_STEP:
                        got[m][(t, f)] = d_out[f, t - t0].cpu().numpy()
        herm = lambda V: np.triu(V) + np.triu(V, 1).conj().T   # the library's orientation
        rel = lambda v, r: float(np.linalg.norm(v - r) / np.linalg.norm(r))
        errs = {m: [] for m in methods}
        spans = []
        for t, f in corners:
            V_ref, span, _ = cpu_sample(pool, cores, w, t, f, nsamp=S)
            spans.append(span)
            for m in methods:
                errs[m].append({"lst_index": t, "mhz": round(float(w["freqs"][f]) / 1e6, 3),
                                "err": rel(got[m][(t, f)], herm(V_ref))})
        line["rel_err_vs_fp64"] = {
            **{m: max(e["err"] for e in errs[m]) for m in methods},
            "per_slice": errs,
            "bound": {"tc": 1e-4, "tc_fp16": 1e-4, "plain": 1e-5},
            "sample": f"whole slices ({N} ant x {S} src) at (LST index, channel) "
                      f"{[(t, f) for t, f in corners]} of outputs of the timed call shape, against "
                      f"the FP64 oracle of the same inputs; the headline key is the largest"}
        _, span32, nsamp32 = cpu_sample(pool, cores, w, 0, 0, "float32")
        line["cpu_baseline"] = {
            "value": cpu_rate(span32, nsamp32, N, S), "unit": "vis/s", "cores": cores,
            "kind": "port",
            "value_fp64": cpu_rate(min(spans), S, N, S),
            "sample": f"value: the oracle port in float32 (the reference's default precision 1) "
                      f"on {nsamp32} sources of one slice on {cores} processes, extrapolated "
                      f"linearly to {S}; value_fp64: the float64 oracle of one whole slice "
                      f"({S} sources) on {cores} processes"}

    leg = run_leg

    # ---- the small and array-scale configurations ---------------------------
    if rank == 0 and not args.no_configs:
        line["configs"] = leg(run_configs, args, local, pool, cores)

    # ---- batched form: many uneven simulations in one plan ----------------
    if rank == 0 and args.batch_sims > 0:
        line["batch"] = leg(run_batch, args, local)

    # ---- the 2-D median filter (hera_gpu.MedianFilter) ---------------------
    if rank == 0 and not args.no_median:
        line["median"] = leg(run_median, args, local)

    # ---- Omnical redundant calibration (hera_gpu.redcal.omnical) -----------
    if rank == 0 and not args.no_omnical:
        line["omnical"] = leg(run_omnical, args, local)

    # ---- serving: Poisson request stream, continuous batching --------------
    if rank == 0 and args.serve_requests > 0:
        line["serve"] = leg(run_serve, args, local, pool)

    if pool is not None:
        pool.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


# The reference's published vis_gpu timings (hera_gpu/tests/speed_test_output.txt:
# 15, 22; hardware unstated): one call of 350 antennas x 314,159 sources x 10
# LSTs took 0.934 s in FP32 and 13.04 s in FP64.
PUBLISHED_SHAPE = dict(nant=350, nsrc=314_159, ntimes=10)
PUBLISHED_S = {1: 0.934, 2: 13.04}


def run_configs(args, device, pool, cores):
    """The other configurations, each form timed through the device entry
    point (inputs resident, CUDA events on the call's stream, one step = one
    call over all of the configuration's LSTs) and once through the drop-in
    vis_gpu with host arrays (copies included); each output's error against
    the FP64 oracle on its first and last LST (whole slices); the oracle
    port on the host cores as the CPU baseline.

      small      16 antennas, 1000 sources, 10 LSTs, 31x31 Gaussian beams,
                 150 MHz
      array      350 antennas, 100,000 sources, 60 LSTs, 63x63 Airy beams,
                 150 MHz, FP32 (plain and tensor-core) and FP64
      published  the shape of the reference's own timings (350 x 314,159 x
                 10 LSTs, 63x63 Airy beams, 150 MHz), beside its published
                 seconds per call (other, unstated hardware)"""
    import numpy as np
    import torch
    from hera_gpu_gb300 import _native, synth, vis_gpu
    from oracle import vis_oracle
    dev = torch.device("cuda", device)
    ctx = _native.Context(device)
    stream = torch.cuda.Stream(dev)
    small = synth.config_small(seed=0)
    arr = synth.config_array(seed=2, nant=350, nsrc=100_000, ntimes=60, nfreq=1, fmin=150e6,
                             fmax=150e6, P=63)
    arr["bm_cubes"] = synth.beams_for(arr, dtype=np.float64)
    pub = synth.config_array(seed=3, nfreq=1, fmin=150e6, fmax=150e6, P=63, **PUBLISHED_SHAPE)
    pub["bm_cubes"] = synth.beams_for(pub, dtype=np.float64)
    forms = [("plain", 1), ("tc", 1), ("tc_fp16", 1), ("plain", 2)]
    plan = {"small": (small, 20, 3), "array": (arr, 3, 1), "published": (pub, 2, 1)}
    out = {}
    for name, (c, steps, warm) in plan.items():
        N, S, T = c["antpos"].shape[0], c["crd_eq"].shape[1], c["eq2tops"].shape[0]
        freq = float(c["freqs"][0])
        res = {"nant": N, "nsrc": S, "ntimes": T, "beam_px": c["bm_cubes"].shape[-1],
               "mhz": freq / 1e6, "forms": {}}
        refs = {}
        for method, prec in forms:
            rt = np.float32 if prec == 1 else np.float64
            ct = torch.complex64 if prec == 1 else torch.complex128
            host = {k: np.ascontiguousarray(c[k], dtype=rt)
                    for k in ("antpos", "eq2tops", "crd_eq", "I_sky")}
            host["bm"] = np.ascontiguousarray(c["bm_cubes"], dtype=rt)
            d = {k: torch.from_numpy(v).to(dev) for k, v in host.items()}
            o = torch.empty((1, T, N, N), dtype=ct, device=dev)
            n_steps = 1 if prec == 2 and name != "small" else steps

            def call():
                ctx.vis_multifreq_device(prec, method, d["antpos"].data_ptr(), N, [freq],
                                         d["eq2tops"].data_ptr(), T, d["crd_eq"].data_ptr(),
                                         d["I_sky"].data_ptr(), S, d["bm"].data_ptr(),
                                         host["bm"].shape[-1], o.data_ptr(), stream.cuda_stream)
            for _ in range(warm):
                call()
            torch.cuda.synchronize(dev)
            ctx.sync()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(n_steps):
                call()
            e1.record(stream)
            torch.cuda.synchronize(dev)
            ctx.sync()
            ms = e0.elapsed_time(e1) / n_steps
            t0 = time.perf_counter()
            V = vis_gpu(host["antpos"], freq, host["eq2tops"], host["crd_eq"], host["I_sky"],
                        host["bm"][0], precision=prec, method=method, context=ctx)
            e2e_s = time.perf_counter() - t0
            key = method if method.startswith("tc") else f"{method}_fp{32 * prec}"
            form = {"ms_per_call": ms, "vis_per_s": T * N * N / (ms / 1e3),
                    "e2e_vis_per_s": T * N * N / e2e_s, "steps": n_steps}
            if name == "published":
                form["reference_published_s"] = PUBLISHED_S[prec]
            # error on the first and last LST against the FP64 oracle of the
            # inputs as the GPU saw them
            errs = []
            for t in (0, T - 1):
                rk = (prec, t)
                if rk not in refs:
                    seen = {k: np.asarray(v, dtype=np.float64) for k, v in host.items()}
                    if pool is not None and S > 20000:
                        ws = dict(antpos=seen["antpos"], freqs=np.array([freq]),
                                  eq2tops=seen["eq2tops"], crd_eq=seen["crd_eq"],
                                  I_sky=seen["I_sky"], bm_cubes=seen["bm"])
                        Vr = cpu_sample(pool, cores, ws, t, 0, nsamp=S)[0]
                        refs[rk] = np.triu(Vr) + np.triu(Vr, 1).conj().T
                    else:
                        refs[rk] = vis_oracle(seen["antpos"], freq, seen["eq2tops"][t:t + 1],
                                              seen["crd_eq"], seen["I_sky"], seen["bm"][0])[0]
                ref = refs[rk]
                errs.append(float(np.linalg.norm(V[t] - ref) / np.linalg.norm(ref)))
            form["rel_err_vs_fp64"] = max(errs)
            res["forms"][key] = form
        # the oracle port on the host cores, float32 and float64
        if pool is not None:
            cpu = {}
            for dt in ("float32", "float64"):
                ws = dict(antpos=c["antpos"], freqs=np.array([freq]), eq2tops=c["eq2tops"],
                          crd_eq=c["crd_eq"], I_sky=c["I_sky"], bm_cubes=c["bm_cubes"])
                _, span, nsamp = cpu_sample(pool, cores, ws, 0, 0, dt,
                                            nsamp=min(S, cores * CPU_SAMPLE_SRC))
                cpu[dt] = cpu_rate(span, nsamp, N, S)
            res["cpu_baseline"] = {"vis_per_s_fp32": cpu["float32"], "vis_per_s_fp64": cpu["float64"],
                                   "cores": cores, "kind": "port",
                                   "sample": f"one slice on {cores} processes"
                                             + (", extrapolated linearly in sources"
                                                if S > cores * CPU_SAMPLE_SRC else "")}
        out[name] = res
    return out


# the largest images and windows of the reference's median-filter tests
# (hera_gpu/tests/test_median_filter.py): (rows, cols), (k0, k1)
MEDIAN_CASES = [((7000, 7000), (3, 3)), ((4000, 4000), (5, 5)), ((997, 997), (9, 9)),
                ((8013, 700), (9, 5))]


def run_median(args, device, steps=5, warmup=3):
    """The median filter on the reference's test shapes (uniform random
    images): device time with the image resident (CUDA events around
    hv_median_filter_device), end to end through MedianFilter (host arrays,
    copies included), and scipy.signal.medfilt2d on one host core, the
    reference's own check."""
    import ctypes
    import numpy as np
    import scipy.signal as sps
    import torch
    from hera_gpu_gb300 import MedianFilter, _native
    dev = torch.device("cuda", device)
    ctx = _native.Context(device)
    peaks, _ = load_peaks()
    out = []
    for (rows, cols), (k0, k1) in MEDIAN_CASES:
        img = np.random.default_rng(0).random((rows, cols), dtype=np.float32)
        d_in = torch.from_numpy(img).to(dev)
        d_out = torch.empty_like(d_in)
        stream = torch.cuda.Stream(dev)

        def call():
            ctx.check(ctx.lib.hv_median_filter_device(
                ctx.h, ctypes.c_void_p(d_in.data_ptr()), ctypes.c_void_p(d_out.data_ptr()), 1,
                rows, cols, k0, k1, ctypes.c_void_p(stream.cuda_stream)))
        for _ in range(warmup):
            call()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            call()
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / steps
        MedianFilter(input=img, kernel_size=(k0, k1), context=ctx)
        t0 = time.perf_counter()
        for _ in range(steps):
            MedianFilter(input=img, kernel_size=(k0, k1), context=ctx)
        e2e_s = (time.perf_counter() - t0) / steps
        t0 = time.perf_counter()
        sps.medfilt2d(img, (k0, k1))
        cpu_s = time.perf_counter() - t0
        px = rows * cols
        gbs = 8.0 * px / (ms / 1e3) / 1e9
        out.append({"image": [rows, cols], "window": [k0, k1], "ms": ms,
                    "mpix_per_s": px / (ms / 1e3) / 1e6, "e2e_mpix_per_s": px / e2e_s / 1e6,
                    "hbm_gbs": gbs, "hbm_frac": gbs / peaks.get("hbm_gbs", 6800.0),
                    "cpu_scipy_mpix_per_s": px / cpu_s / 1e6})
    return {"cases": out, "unit": "Mpixel/s", "cpu": "scipy.signal.medfilt2d, 1 host core",
            "bytes_per_pixel": 8, "data": "uniform random float32 images"}


# the configurations of the reference's own omnical timings
# (hera_gpu/redcal.py:431-458: 2000 problems, Quadro T2000, the shipped
# chunk_size = nthreads // 16): (nants, precision, seconds there)
OMNICAL_CASES = [(54, 2, 1.5), (126, 2, 5.2), (180, 2, 9.9), (180, 1, 7.3)]
OMNICAL_NDATA = 2000


def run_omnical(args, device, steps=3, warmup=3, cpu_sample=8):
    """Omnical with the reference's defaults (conv_crit 1e-10, maxiter 50,
    check_every 4, check_after 1, gain 0.3) on 2000 problems of a hex
    redundant array of nants antennas (synthetic: gains 1 + 5% scatter, 1%
    noise, start 2% off).  Device time with the inputs resident (CUDA events
    around the reset of the starting point and hv_omnical_device), end to
    end through the drop-in omnical (host arrays, copies included), and the
    oracle on a sample of problems on one host core, extrapolated."""
    import ctypes
    import numpy as np
    import torch
    from hera_gpu_gb300 import _native, omnical, synth
    from oracle import omnical_oracle
    dev = torch.device("cuda", device)
    ctx = _native.Context(device)
    out = []
    cases = OMNICAL_CASES
    if args.omnical_cases:
        want = [tuple(int(x) for x in c.split(":")) for c in args.omnical_cases.split(",")]
        pub = {(n, p): r for n, p, r in OMNICAL_CASES}
        cases = [(n, p, pub.get((n, p))) for n, p in want]
    for nants, precision, ref_s in cases:
        ggu, nubls = synth.hex_redundant_layout(nants)
        nbls = len(ggu)
        g0, u0, d, w = synth.redundant_data(ggu, nubls, OMNICAL_NDATA, seed=nants, noise=0.01)
        ct, rt = (np.complex64, np.float32) if precision == 1 else (np.complex128, np.float64)
        g0, u0, d, w = g0.astype(ct), u0.astype(ct), d.astype(ct), w.astype(rt)
        t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev)
             for k, v in (("g0", g0), ("u0", u0), ("d", d), ("w", w))}
        tg, tu = torch.empty_like(t["g0"]), torch.empty_like(t["u0"])
        tc, tv = torch.empty(OMNICAL_NDATA, dtype=t["w"].dtype, device=dev), \
            torch.empty(OMNICAL_NDATA, dtype=t["w"].dtype, device=dev)
        ti = torch.empty(OMNICAL_NDATA, dtype=torch.int32, device=dev)
        stream = torch.cuda.Stream(dev)
        vp = lambda x: ctypes.c_void_p(x.data_ptr())

        def call():
            with torch.cuda.stream(stream):
                tg.copy_(t["g0"])
                tu.copy_(t["u0"])
            ctx.check(ctx.lib.hv_omnical_device(
                ctx.h, precision, ggu.ctypes.data_as(ctypes.c_void_p), nbls, vp(tg), nants,
                vp(tu), nubls, vp(t["d"]), vp(t["w"]), OMNICAL_NDATA, 1e-10, 50, 4, 1, 0.3,
                vp(tc), vp(ti), vp(tv), ctypes.c_void_p(stream.cuda_stream)))
        for _ in range(warmup):
            call()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            call()
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / steps
        iters = ti.cpu().numpy()
        omnical(ggu, g0, u0, d, w, precision=precision, context=ctx)
        t0 = time.perf_counter()
        for _ in range(steps):
            res = omnical(ggu, g0, u0, d, w, precision=precision, context=ctx)
        e2e_s = (time.perf_counter() - t0) / steps
        case = {"nants": nants, "nbls": nbls, "nubls": nubls, "precision": precision,
                "problems": OMNICAL_NDATA, "ms": ms, "problems_per_s": OMNICAL_NDATA / (ms / 1e3),
                "e2e_s": e2e_s, "mean_iters": float(iters.mean()),
                "reference_published_s": ref_s}
        if not args.no_cpu:
            t0 = time.perf_counter()
            ref = omnical_oracle(ggu, g0[:cpu_sample], u0[:cpu_sample], d[:cpu_sample],
                                 w[:cpu_sample], precision=precision)
            case["cpu_oracle_s_extrapolated"] = \
                (time.perf_counter() - t0) / cpu_sample * OMNICAL_NDATA
            scale = float(np.abs(ref["gains"]).max())
            case["max_gain_diff_vs_oracle"] = \
                float(np.abs(res["gains"][:cpu_sample] - ref["gains"]).max() / scale)
            case["iters_equal_vs_oracle"] = \
                float((res["iters"][:cpu_sample] == ref["iters"]).mean())
        out.append(case)
    return {"cases": out, "data": "synthetic hex redundant arrays, 1% noise",
            "reference_published": "hera_gpu/redcal.py:431-458, Quadro T2000, other hardware",
            "cpu": f"oracle (numpy, 1 process) on {cpu_sample} problems, extrapolated"}


def run_batch(args, device, steps=5, warmup=3):
    """The batched-form configuration: --batch-sims simulations with nant
    log-uniform in [16, 350] on random hex subsets, nsrc log-uniform in
    [1e3, 2e5], ntimes uniform in [1, 60], nfreq uniform in [1, 16] over
    100-200 MHz and beams of 31 or 63 pixels, planned as one batch (one
    persistent fused launch per cluster class), split-K tuned on the batch,
    captured as a CUDA graph and replayed.  Inputs are resident on the
    device; a step is one replay, and its time includes every kernel of the
    batch (source sort, preparation, fused launches, reductions)."""
    import numpy as np
    import torch
    from hera_gpu_gb300 import _native, synth
    dev = torch.device("cuda", device)
    specs = synth.config_batch(seed=0, nsims=args.batch_sims)
    keep, sims = [], []
    herk_flops = 0.0   # algorithmic: 4 N (N + 1) per source above the horizon, per slice
    for sp in specs:
        arrs, dish = synth.make_sim_arrays(sp)
        e2t = np.asarray(arrs["eq2tops"], dtype=np.float32).astype(np.float64)
        crd = np.asarray(arrs["crd_eq"], dtype=np.float32).astype(np.float64)
        up = sum(int(np.count_nonzero(e2t[t][2] @ crd > 0)) for t in range(sp["ntimes"]))
        herk_flops += 4.0 * sp["nant"] * (sp["nant"] + 1) * up * sp["nfreq"]
        d = {k: torch.from_numpy(np.ascontiguousarray(arrs[k])).to(dev)
             for k in ("antpos", "eq2tops", "crd_eq", "I_sky")}
        # Airy power beams (2 J1(x)/x)^2, x = pi D sin(theta) / lambda, as
        # synth.airy_beams, evaluated on the device
        g = torch.linspace(-1.0, 1.0, sp["P"], dtype=torch.float64, device=dev)
        st = torch.clamp(torch.hypot(g[None, :], g[:, None]), max=1.0)
        dsh = torch.from_numpy(dish).to(dev)
        lam = synth.C_LIGHT / torch.from_numpy(arrs["freqs"]).to(dev)
        x = torch.pi * dsh[None, :, None, None] * st[None, None] / lam[:, None, None, None]
        safe = torch.where(x == 0, torch.ones_like(x), x)
        bm = torch.where(x == 0, torch.ones_like(x), (2 * torch.special.bessel_j1(safe) / safe) ** 2)
        d["bm_cubes"] = bm.to(torch.float32).contiguous()
        d["out"] = torch.empty((len(arrs["freqs"]), sp["ntimes"], sp["nant"], sp["nant"]),
                               dtype=torch.complex64, device=dev)
        keep.append(d)
        sims.append(dict(antpos=d["antpos"].data_ptr(), eq2tops=d["eq2tops"].data_ptr(),
                         crd_eq=d["crd_eq"].data_ptr(), I_sky=d["I_sky"].data_ptr(),
                         bm_cubes=d["bm_cubes"].data_ptr(), freqs=arrs["freqs"],
                         vis_out=d["out"].data_ptr(), nant=sp["nant"], ntimes=sp["ntimes"],
                         nsrc=sp["nsrc"], beam_px=sp["P"]))
    torch.cuda.synchronize(dev)
    ctx = _native.Context(device)
    t0 = time.perf_counter()
    b = _native.Batch(ctx, sims, graph=True, autotune=True)
    plan_s = time.perf_counter() - t0
    stream = torch.cuda.Stream(dev)
    for _ in range(warmup):
        b.launch(stream.cuda_stream)
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        b.launch(stream.cuda_stream)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    b.sync()
    vis = sum(sp["nfreq"] * sp["ntimes"] * sp["nant"] ** 2 for sp in specs)
    peaks, peak_src = load_peaks()
    peak = peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops"))
    achieved = herk_flops / (ms / 1e3) / 1e12
    out = {"sims": len(specs), "vis_per_step": vis, "ms_per_step": ms,
           "vis_per_s": vis / (ms / 1e3), "unit": "vis/s", "steps": steps, "warmup": warmup,
           "graph": True, "autotune": True, "plan_s": plan_s,
           "gpu_launches_per_step": b.launches,
           "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak,
                        "unit": "TFLOP/s", "frac": achieved / peak,
                        "peak_kind": f"bf16 dense sustained ({peak_src})",
                        "algorithmic": "4 N (N+1) per source above the horizon, per slice, "
                                       "summed over the batch, over the whole replay time "
                                       "(preparation, fused launches and reductions)"},
           "workload": "nant logU[16,350] hex subsets, nsrc logU[1e3,2e5], ntimes U[1,60], "
                       "nfreq U[1,16] 100-200 MHz, P in {31,63}; inputs resident"}
    b.close()
    del keep
    torch.cuda.empty_cache()
    return out


def run_serve(args, device, pool):
    """The serving configuration: Poisson arrivals at --serve-rate of requests
    from the batched-form size distribution plus 5 % large requests (350
    antennas, 1M sources, 60 LSTs), 8 resident beam/layout sets, HBM budget
    150 GB, --serve-slots slots of at most --serve-max-batch requests.
    Latency = arrival to result in host memory.  A second run at
    --serve-rate-low shows the latency below saturation."""
    import numpy as np
    from hera_gpu_gb300 import _native, serve
    ctxs = [_native.Context(device) for _ in range(args.serve_slots)]
    specs, reqs = serve.workload(args.serve_requests, rate_hz=args.serve_rate, seed=7)
    sets = serve.build_sets(ctxs[0], specs, nfreq=16)
    srv = serve.Server(sets, ctxs, hbm_budget=150e9, max_batch=args.serve_max_batch)
    # page-locked staging sized up front, and the plan/launch path warmed
    # once (first-use costs are not steady state)
    srv.reserve(reqs)
    warm = serve.workload(4, rate_hz=1e4, large_frac=0.0, seed=99)[1]
    srv.run(warm)

    # the oracle sample: 1 % of the small requests, one (time, channel) slice
    # each, kept by the result consumer (the other results are delivered and
    # dropped, as a service hands them on)
    rng = np.random.default_rng(3)
    small_ids = [r.rid for r in reqs if r.nsrc < 100_000]
    sample_ids = set(rng.choice(small_ids, size=max(1, len(reqs) // 100), replace=False).tolist())
    kept = {}

    def consume(r, view):
        if r.rid in sample_ids:
            kept[r.rid] = view[0, 0].copy()

    def one_run(rs, keep):
        done = srv.run(rs, on_result=consume if keep else (lambda r, v: None))
        out = serve.summarize(done, max(r.t_done for r in done))
        out["offered_req_per_s"] = len(rs) / max(r.arrival for r in rs)
        return done, out

    done, out = one_run(reqs, True)
    out.update({"rate_hz": args.serve_rate, "large_frac": 0.05, "slots": len(ctxs),
                "max_batch": args.serve_max_batch, "resident_sets": len(sets),
                "hbm_budget_gb": 150,
                "latency": "arrival to result in host memory (page-locked staging, handed to a "
                           "consumer callback)"})
    if args.serve_rate_low > 0:
        _, reqs_low = serve.workload(args.serve_requests, rate_hz=args.serve_rate_low, seed=7)
        _, low = one_run(reqs_low, False)
        out["at_lower_rate"] = {k: low[k] for k in ("offered_req_per_s", "p50_ms", "p99_ms",
                                                    "p99_first_half_ms", "p99_second_half_ms",
                                                    "mean_ms", "vis_per_s", "wall_s", "served")}
        out["at_lower_rate"]["rate_hz"] = args.serve_rate_low
    # error vs the FP64 oracle on a 1 % sample (one (time, channel) slice of
    # each sampled small request; the checker runs in the host-process pool)
    if pool is not None:
        errs = []
        for r in done:
            if r.rid not in kept:
                continue
            sp = specs[r.set_id]
            g = np.random.default_rng(sp["seed"])
            full = serve.synth.hex_array(350, 14.6, 0.01, g)
            sel = np.sort(g.choice(350, size=sp["nant"], replace=False))
            dish = 14.0 * (1.0 + 0.02 * g.uniform(-1.0, 1.0, sp["nant"]))
            f0 = sets[r.set_id].freqs[0]
            bm = serve.synth.airy_beams(sp["nant"], sp["P"], f0, dish).astype(np.float32)
            ant = full[sel].astype(np.float32).astype(np.float64)
            V = pool.apply(_cpu_worker, ((ant, float(f0), r.eq2tops[0].astype(np.float64),
                                          r.crd_eq.astype(np.float64),
                                          r.I_sky.astype(np.float64), bm,
                                          np.dtype(np.float64)),))[0]
            errs.append(float(np.linalg.norm(kept[r.rid] - V) / max(np.linalg.norm(V), 1e-300)))
        out["sample_rel_err_max"] = max(errs)
        out["sample"] = f"{len(errs)} requests, slice (t=0, {sets[0].freqs[0] / 1e6:.0f} MHz)"
    for st in sets:
        st.close()
    return out


def main():
    args = parse_args()
    rc = launch_replicas(args)
    if rc is not None:
        return rc
    if args.dry_run:
        return run_dry(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.serve_only:
        print(json.dumps({"serve": run_serve(args, 0, None)}), flush=True)
        return 0
    if args.batch_only:
        print(json.dumps({"batch": run_batch(args, 0)}), flush=True)
        return 0
    if args.median_only:
        print(json.dumps({"median": run_median(args, 0)}), flush=True)
        return 0
    if args.omnical_only:
        print(json.dumps({"omnical": run_omnical(args, 0)}), flush=True)
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
