"""bench.py under torchrun with N > 1 GPUs runs N independent replicas ("replicas only": a single
scene does not shard without halo exchanges every solver iteration).  The data path has no
collective; the ranks meet only for the barrier around the timed region and the max over ranks
of the timed seconds.  These tests run that host logic as world-size-2 gloo ranks on the CPU:
  * max_over_ranks returns the slowest rank's time on every rank, and replica_rate the whole-job
    rate from it;
  * the reference arm on a rank other than 0 exits 0 without work and prints nothing.
"""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = 1.0 + 0.25 * rank                    # the ranks' timed seconds
    t_max = bench.max_over_ranks(t, dist, "cpu")
    dist.barrier()
    out[rank] = (t_max, bench.replica_rate(world, 1000, 20, t_max))
    dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate_with_two_gloo_ranks():
    import torch.multiprocessing as mp
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 1.25
    assert res[0][1] == res[1][1] == pytest.approx(2 * 1000 * 20 / 1.25)


def test_without_process_group_the_time_is_the_rank_own():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.replica_rate(1, 1_048_576, 20, 0.2) == pytest.approx(1_048_576 * 100)


def test_reference_arm_on_a_nonzero_rank_does_no_work():
    env = {**os.environ, "RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "20", "--warmup", "5"], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
