"""Host logic of the N > 1 bench path on CPU (gloo, world size 2).

The FDM step does not shard: `bench.py --gpus N` under torchrun runs N independent
replicas, takes the slowest replica's time (max over ranks) and reports the whole-job
rate N x units / that time.  The reference arm runs on rank 0 only; other ranks exit 0
without work."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, str(ROOT))
    import bench
    t = 1.5 + rank  # rank 1 is the slow replica
    tmax = bench.max_over_ranks(t, dist, "cpu")
    rate = bench.whole_job_rate(world, 1000, tmax)
    dist.barrier()
    q.put((rank, tmax, rate))
    dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [2.5, 2.5]          # every rank sees the slowest time
    assert [o[2] for o in out] == [800.0, 800.0]      # 2 replicas x 1000 units / 2.5 s


def test_sweep_sharding_is_a_balanced_partition():
    """The sweep's cost-balanced sharding: every film on exactly one rank, rank costs
    within a few percent of each other (n log2 n of the 4 x 384 seeded films)."""
    sys.path.insert(0, str(ROOT))
    import numpy as np
    import bench
    rng = np.random.default_rng(1)
    cells = [int(rng.integers(16, 257)) * int(rng.integers(16, 129)) * int(rng.choice([1, 2, 4])) for _ in range(1536)]
    costs = [c * np.log2(c) for c in cells]
    parts = bench.shard_by_cost(costs, 4)
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(1536))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) / min(loads) < 1.01
    assert bench.shard_by_cost(costs, 1) == [list(range(1536))]


def test_single_process_helpers():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(3.0, None, "cpu") == 3.0
    assert bench.whole_job_rate(1, 500, 2.0) == 250.0


def test_reference_arm_runs_on_rank0_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload",
                        "box_64x32x4_heun", "--steps", "1", "--warmup", "0"],
                       capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""
    env = dict(os.environ, RANK="0", WORLD_SIZE="2", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload",
                        "box_64x32x4_heun", "--steps", "1", "--warmup", "0"],
                       capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["cpu_baseline"]["kind"] == "port"


def test_gpus_flag_launches_ranks_itself():
    """`bench.py --gpus 2` started as one plain process launches two ranks itself
    (torch.distributed.run on 127.0.0.1); with --impl reference rank 0 alone works and
    prints one line for the whole job."""
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--gpus", "2", "--impl", "reference",
                        "--workload", "box_64x32x4_heun", "--steps", "1", "--warmup", "0"],
                       capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.strip().splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["config"]["same_grid"] is True
