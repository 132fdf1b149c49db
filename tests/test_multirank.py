"""The bench's multi-GPU path on the host: two ranks over gloo (127.0.0.1)
reduce their step times to the slowest rank's and report the whole-job
rate; under a launcher, the reference arm runs on rank 0 alone and the other
ranks leave without work.  Replicas only: the path does not shard, so no
collective touches the data."""
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        times = bench.max_over_ranks([1.0 + rank, 5.0 - rank, 2.5], world)
        rate = bench.whole_job_rate(1000, 10, world, times[0])
        out.put((rank, times, rate))
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time_and_sum_the_work():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict()
    for _ in range(2):
        r, times, rate = q.get(timeout=120)
        got[r] = (times, rate)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        times, rate = got[r]
        assert times == [2.0, 5.0, 2.5]
        assert rate == 2 * 1000 * 10 / 2e-3


def test_single_process_keeps_its_times():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([3.0, 4.0], 1) == [3.0, 4.0]


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
