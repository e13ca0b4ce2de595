"""The N-GPU replica path on CPU: two gloo ranks aggregate throughput over
the slowest rank, and the reference arm's other ranks exit without work."""
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    from omega_h_gb300.replicas import max_over_ranks, replica_throughput, world_size
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        assert world_size() == world
        secs = 1.0 + rank          # rank 1 is the slowest
        value, s = replica_throughput(10.0, secs)
        out[rank] = (value, s, max_over_ranks(-rank))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_over_the_slowest():
    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    for r in range(2):
        value, s, m = out[r]
        assert s == 2.0 and value == pytest.approx(2 * 10.0 / 2.0) and m == 0.0


def test_single_process_is_its_own_max():
    sys.path.insert(0, ROOT)
    from omega_h_gb300.replicas import replica_throughput
    assert replica_throughput(5.0, 0.5) == (10.0, 0.5)


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1",
               MASTER_ADDR="127.0.0.1", MASTER_PORT=str(_free_port()))
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
