"""Multi-process paths of bench.py on CPU (gloo): the replicas' step time is the
slowest rank's, every rank agrees on it, the whole-job throughput counts all
replicas, and under torchrun the reference arm runs on rank 0 only."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    got = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, got))


def test_step_time_is_the_slowest_rank_on_every_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29511
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = dict(q.get(timeout=10) for _ in range(2))
    assert res == {0: 15.0, 1: 15.0}


def test_throughput_counts_every_replica():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_throughput(1000, 1, 1.0) == pytest.approx(1e6)
    assert bench.job_throughput(1000, 4, 2.0) == pytest.approx(2e6)
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5


@pytest.mark.parametrize("mode", [["--impl", "reference"], ["--serve"], ["--batch"]])
def test_nonzero_ranks_exit_without_work(mode):
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *mode], env=env,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
