"""The multi-GPU bench path runs one replica per rank: the ranks exchange
nothing but the barrier and the max-over-ranks time.  Those, the whole-job
rate and the per-rank workloads are checked here on two CPU ranks (gloo)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(1.0 + rank, world, "cpu")     # rank 1 is the slower one
    rate = bench.whole_job_rate(1000, 10, world, t)
    dist.barrier()
    out[rank] = (t, rate)
    dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time_and_sum_the_replicas():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, join=True,
                       start_method="spawn")
    assert out[0] == out[1]
    t, rate = out[0]
    assert t == 2.0 and rate == world * 1000 * 10 / 2.0


def test_replicas_differ_per_rank():
    sys.path.insert(0, ROOT)
    import bench
    from sop_gb300 import system
    ns, _ = system.ensemble_spec(bench.N_TRAJ, 60, 1500, 0.5, 0.8, seed=4)
    # molecule k of rank r has structure seed r * N_TRAJ + k
    a = system.generate(int(ns[0]), 0 * bench.N_TRAJ + 0)
    b = system.generate(int(ns[0]), 1 * bench.N_TRAJ + 0)
    assert a.n == b.n and not (a.xyz == b.xyz).all()
