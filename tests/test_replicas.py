"""Replicas-only multi-GPU timing of bench.py on CPU: two gloo ranks agree on
the slowest rank's time and the whole-job throughput; the reference arm's
non-zero ranks exit without work."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out):
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=2)
    try:
        out[rank] = bench.job_throughput([10.0, 20.0][rank], 5, 2, "cpu")
    finally:
        dist.destroy_process_group()


def test_job_throughput_two_gloo_ranks():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(port, out), nprocs=2, join=True)
        res = dict(out)
    # both ranks: 2 replicas x 5 steps over the slower rank's 20 ms
    assert res[0] == res[1] == (500.0, 20.0)


def test_job_throughput_single_rank():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_throughput(12.5, 20, 1) == (1600.0, 12.5)


def test_reference_arm_nonzero_rank_exits_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1",
                          "--warmup", "0", "--workload", "m21_n1k"], cwd=ROOT, env=env,
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip() == ""
