"""The multi-GPU path is replicas only: every rank factors its own instance
and the job's time is the slowest rank's.  The host side of that is checked
here with two gloo ranks on the CPU: the max-over-ranks reduction, the
whole-job throughput, and the reference arm under torchrun (rank 0 alone runs
and prints one line; the other rank exits 0 without work)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 10.0 + 5.0 * rank            # rank 1 is the slower one
    m = bench.max_over_ranks(ms, dist, "cpu")
    v = bench.replica_throughput(1e12, world, m)
    out.put((rank, m, v))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_throughput_with_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29400 + os.getpid() % 1000
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=120)
        assert p.exitcode == 0
    for rank, m, v in res:
        assert m == 15.0                       # both ranks see the slowest time
        assert abs(v - 2 * 1e12 / 15e-3 / 1e12) < 1e-9


def test_reference_arm_under_torchrun_prints_once():
    port = 29500 + os.getpid() % 1000
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl",
           "reference", "--workload", "ns3_nt3_nd2", "--gpus", "2", "--steps", "1", "--warmup",
           "0", "--ref-seconds", "0.05"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
