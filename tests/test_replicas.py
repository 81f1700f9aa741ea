"""The multi-process (replica) path of bench.py on the CPU: world size 2 over
gloo, each rank a replica with its own timing. Checks the max-over-ranks
reduction that the timing rule uses and the whole-job value, and that every
rank draws a different ensemble (rank = seed) of the same shape."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        from fluids2d_gb300 import workloads as wl
        ms = 10.0 + 5.0 * rank  # the slower replica is rank 1
        mx = bench.max_over_ranks(ms, world)
        members = wl.ensemble_case(count=8, seed=rank)
        cells = sum(c["nx"] * c["ny"] for c in members)
        sig = float(sum(np.abs(c["fields"]["omega"]).sum() for c in members))
        t = torch.tensor([float(cells), sig], dtype=torch.float64)
        allt = [torch.zeros(2, dtype=torch.float64) for _ in range(world)]
        dist.all_gather(allt, t)
        out[rank] = (mx, bench.replica_value(1000, 4, mx, world),
                     [tuple(x.tolist()) for x in allt])
    finally:
        dist.destroy_process_group()


def test_replica_timing_and_value_over_gloo():
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as man:
        out = man.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        mx, value, gathered = res[r]
        assert mx == 15.0
        assert value == pytest.approx(world * 1000 * 4 / 0.015)
        # distinct ensembles per rank (seed = rank), both non-empty
        assert gathered[0][0] > 0 and gathered[1][0] > 0
        assert gathered[0] != gathered[1]


def test_max_over_ranks_single_process():
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.replica_value(100, 2, 10.0, 1) == pytest.approx(2e4)
