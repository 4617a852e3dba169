"""The multi-replica path of bench.py on CPU: two gloo ranks agree on the slowest replica's
time and on the whole-job throughput; the reference arm's non-zero ranks exit without work."""
import os
import socket
import subprocess
import sys

import pytest

from conftest import REPO

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, str(REPO))
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        local = [0.25, 0.5][rank]
        t = bench.max_over_ranks(local, dist, device="cpu")
        q.put((rank, t, bench.job_gbs(world, 10**9, t)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [g[1] for g in got] == [0.5, 0.5]
    assert [g[2] for g in got] == [4.0, 4.0]  # 2 replicas x 1 GB / 0.5 s


def test_single_rank_is_its_own_max():
    sys.path.insert(0, str(REPO))
    import bench
    assert bench.max_over_ranks(1.5) == 1.5


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "1"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
