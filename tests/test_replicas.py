"""The multi-process (replica) path of bench.py on the CPU: world size 2 over
gloo, each rank a replica with its own timing. Checks the max-over-ranks
reduction that the timing rule uses and the whole-job value, that every
rank draws a different ensemble (rank = seed) of the same shape, and runs
the ensemble bench function itself at world size 2 with its GPU calls
replaced by fakes (the path stays unmeasured on more than one GPU)."""
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


# ---- the replica bench path itself, GPU calls replaced by fakes ----------------
class _FakeEvent:
    """CUDA event stand-in: elapsed_time gives a fixed per-step time that
    depends on the rank (rank 1 is the slower replica)."""
    step_ms = 1.0

    def __init__(self, enable_timing=True):
        pass

    def record(self, stream=None):
        pass

    def elapsed_time(self, other):
        return _FakeEvent.step_ms


class _FakeStream:
    cuda_stream = 0


class _FakeEnsemble:
    def __init__(self, members):
        self.members = members
        self._h = object()
        self.n = 0

    def autotune(self, reps=2):
        return {"tile_rows": 64, "sweeps": 2, "tol_in": 1e-6, "ms_per_solve": 1.0}

    def sync(self):
        pass

    def stats(self):
        self.n += 1
        k = self.n
        return dict(cells=0, poisson_iters=100 * k, loop_iters=10 * k, launches_per_step=7,
                    launches_per_iter=20, refine_rounds=5 * k)

    def packed_size(self):
        return sum((c["ny"] + 6) * (c["nx"] + 6) for c in self.members)

    def get_field(self, b, name):
        c = self.members[b]
        return np.zeros((c["ny"] + 6, c["nx"] + 6))


class _FakeLib:
    """The C ABI calls of the ensemble bench: success, fixed timings."""

    def __getattr__(self, name):
        def call(*args):
            if name == "f2d_ensemble_time_stage":
                args[4]._obj.value = 0.25
            if name == "f2d_ensemble_time_solver":
                args[3]._obj.value = 0.125
                args[4]._obj.value = 1000
                args[5]._obj.value = 4
            return 0
        return call


def _bench_worker(rank, world, port, out):
    import contextlib
    import io
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    os.environ["RANK"], os.environ["WORLD_SIZE"] = str(rank), str(world)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        import fluids2d_gb300._lib as _l
        _FakeEvent.step_ms = 2.0 + rank  # rank 1: 3 ms per step
        torch.cuda.set_device = lambda d: None
        torch.cuda.Stream = _FakeStream
        torch.cuda.set_stream = lambda s: None
        torch.cuda.synchronize = lambda *a: None
        torch.cuda.Event = _FakeEvent
        real_empty = torch.empty

        def fake_empty(*a, device=None, pin_memory=False, **k):
            return real_empty(*a, **k)
        torch.empty = fake_empty
        bench._ensemble_make = lambda prec, members, stream: _FakeEnsemble(members)
        _l.lib = lambda: _FakeLib()
        args = bench.argparse.Namespace(workload="ensemble256_fp32", steps=4, warmup=3,
                                        no_autotune=False, no_fp64_form=True,
                                        no_cpu_baseline=True, gpus=world)
        buf = io.StringIO()
        with contextlib.redirect_stdout(buf):
            bench.run_gpu_ensemble(args, rank, world)
        out[rank] = buf.getvalue()
    finally:
        dist.destroy_process_group()


def test_replica_bench_path_over_gloo():
    """run_gpu_ensemble at world size 2 (gloo, GPU calls faked): every rank
    draws its own ensemble (seed = rank), times its steps, the max over ranks
    decides, and rank 0 alone prints one JSON line whose value is the
    whole-job rate of both replicas."""
    import json
    from fluids2d_gb300 import workloads as wl
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as man:
        out = man.dict()
        mp.spawn(_bench_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[1].strip() == ""  # only rank 0 prints
    lines = [ln for ln in res[0].splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    members = wl.ensemble_case(seed=0)
    cells = sum(c["nx"] * c["ny"] for c in members)
    ms = 4 * 3.0  # 4 timed steps of the slower replica
    assert d["n_gpus"] == 2 and d["steps"] == 4 and d["warmup"] == 3
    assert d["config"]["parallelism"] == "replicas x2"
    assert d["config"]["members"] == 256 and d["config"]["cells"] == cells
    assert d["value"] == pytest.approx(2 * cells * 4 / (ms / 1e3))
    assert d["ms_per_step"] == pytest.approx(3.0)
    assert d["e2e"]["h2d_bytes_per_step"] == sum(
        (c["ny"] + 6) * (c["nx"] + 6) * 8 for c in members)
    assert d["roofline"]["kernel_ms"] == 0.125
