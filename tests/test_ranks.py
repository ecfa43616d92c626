"""Replicas over ranks, on CPU processes (gloo).

The path has no exchange step: N GPUs run N independent replicas, and the
job's rate is the units of all ranks over the slowest rank's time.  These
tests run the rank logic of bench.py with world size 2 on the gloo backend,
and the reference arm under torchrun (rank 0 alone reports).
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(1.0 + rank)   # rank 1 is the slow one
        q.put((rank, t, bench.job_rate(100.0, world, t)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_job_rate_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # every rank sees the slowest rank's time; the rate counts both ranks' units
    assert [o[1] for o in out] == [2.0, 2.0]
    assert [o[2] for o in out] == [100.0, 100.0]


def test_max_over_ranks_without_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.job_rate(10.0, 1, 2.0) == 5.0


def test_reference_arm_under_torchrun_reports_once():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(30500 + os.getpid() % 1000),
           "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
           "--nant", "16", "--nsrc", "2048", "--nfreq", "2"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    # the same workload description as the GPU arm's (bench.step_config),
    # and a step time that is the measured sample's, not an extrapolation
    import argparse
    sys.path.insert(0, ROOT)
    import bench
    assert line["config"] == bench.step_config(argparse.Namespace(nant=16, nsrc=2048, nfreq=2), 2)
    assert line["dtype"] == "f32" and line["cpu_baseline"]["value_fp64"] > 0
    assert line["ms_per_step"] < 60e3


def test_gpus_flag_launches_the_replicas_itself():
    # `bench.py --gpus 2` outside torchrun starts two ranks through
    # torch.distributed.run; the dry run needs no GPU (gloo), and the line
    # reports both ranks and the slowest rank's time
    r = subprocess.run([sys.executable, "bench.py", "--gpus", "2", "--dry-run"], cwd=ROOT,
                       capture_output=True, text=True, timeout=600,
                       env={k: v for k, v in os.environ.items()
                            if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")})
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["n_gpus"] == 2 and line["dry_run"]
    assert line["ms_per_step"] >= 20.0          # rank 1 sleeps 20 ms
    assert line["config"]["parallelism"] == "replicas x2"

