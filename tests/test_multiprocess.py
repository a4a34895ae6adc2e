"""The N > 1 launch of bench.py (replicas, one process per GPU) on CPU with
a world-size-2 gloo group: the job time is the slowest rank's, the value
counts every replica's pixels, and the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, REPO)
    import argparse
    import contextlib
    import io

    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    got = bench.max_over_ranks(10.0 + rank)
    assert bench._dist_env() == (world, rank, rank)
    buf = io.StringIO()
    rc = None
    if rank != 0:  # rank 0 would run the full CPU workload; the others must not
        with contextlib.redirect_stdout(buf):
            rc = bench.run_reference(argparse.Namespace(steps=1, warmup=3))
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"r{rank}.txt"), "w") as f:
        f.write(f"{got} {rc} {len(buf.getvalue())}")


def test_two_rank_gloo_max_and_rank_gating(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    r0 = open(tmp_path / "r0.txt").read().split()
    r1 = open(tmp_path / "r1.txt").read().split()
    assert float(r0[0]) == 11.0 and float(r1[0]) == 11.0
    assert r1[1] == "0" and r1[2] == "0"  # rank 1: reference arm exits 0, prints nothing


def test_whole_job_value_counts_every_replica():
    sys.path.insert(0, REPO)
    import bench

    one = bench.whole_job_gpx(1, 6 * 4096 * 4096, 10, 30.0)
    two = bench.whole_job_gpx(2, 6 * 4096 * 4096, 10, 30.0)
    assert two == pytest.approx(2 * one)
    assert one == pytest.approx(6 * 4096 * 4096 * 10 / 0.030 / 1e9)
