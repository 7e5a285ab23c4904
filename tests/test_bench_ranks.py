"""The multi-rank (torchrun) logic of bench.py on CPU with the gloo backend:
the job time is the slowest rank's, each rank draws its own streams, and the
reference arm under two ranks prints one line from rank 0 while rank 1 exits
cleanly."""
import json
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(10.0 + 5 * rank, world, device="cpu")
    q.put((rank, t, bench.rank_seed(rank)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_seeds_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29517
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [t for _, t, _ in out] == [15.0, 15.0]
    assert out[0][2] != out[1][2]


def test_reference_arm_two_ranks():
    env = dict(os.environ, OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", "29519", "bench.py", "--impl",
           "reference", "--workload", "dot2", "--gpus", "2", "--steps", "1", "--warmup", "1",
           "--cpu-seconds", "2"]
    r = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["cores"] >= 1
