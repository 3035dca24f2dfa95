"""The multi-rank path of bench.py on CPU (gloo, world size 2): every rank
runs an independent replica, the job's time is the slowest rank's, and the
whole-job throughput adds the ranks' rods; the reference arm runs on rank 0
only."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    seconds = 1.0 + 0.5 * rank  # rank 1 is the slower one
    dist.barrier()
    t = bench.max_over_ranks(torch, dist, world, seconds, "cpu")
    value = bench.job_throughput(world, 100, 10, t)
    out[rank] = (t, value)
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_job_throughput_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert set(res) == {0, 1}
    for rank in range(world):
        t, value = res[rank]
        assert t == 1.5  # the slowest rank's time, seen by every rank
        assert value == pytest.approx(world * 100 * 10 / 1.5)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
