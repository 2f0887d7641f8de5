"""The multi-GPU story of this path is replicas (one independent fit per GPU, no data-path
collective): `bench.py` under torchrun times each rank's fits, takes the slowest rank's step
time, and lets rank 0 alone print.  Its host logic runs here on CPU ranks over gloo."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks(1.5 + rank, dist, device="cpu")
        none = bench.max_over_ranks(None, dist, device="cpu")
        q.put((rank, got, none))
    finally:
        dist.destroy_process_group()


def test_step_time_is_the_slowest_rank_over_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(r for r, _, _ in res) == [0, 1]
    assert all(got == 2.5 and none is None for _, got, none in res)


def test_single_process_keeps_its_own_value():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25) == 3.25


@pytest.mark.parametrize("rank", ["1", "3"])
def test_reference_arm_non_zero_ranks_exit_without_work(rank):
    """`bench.py --impl reference` under torchrun: only rank 0 times the CPU path and prints."""
    env = dict(os.environ, RANK=rank, WORLD_SIZE="4", LOCAL_RANK=rank)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "4"],
                       capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
