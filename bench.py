"""Benchmark of the time-stepping hot path (one JSON line on stdout).

Metric: cell-updates/s = nx*ny*steps / time (the inverse of the reference's
own s/dof printout, model.py:89-93). A benchmark step is one model time step
(SSP-RK3: three fused stage kernels plus their diagnostics, including the
Poisson solves) over the whole grid of every model of the workload.

Default workload (the configuration the headline metric is quoted on): a
batched ensemble of 256 eulerpsi closed basins with sizes drawn from
{64,128,192,256,384,512}^2 and 0-4 islands each, Gaussian-vortex initial
conditions, WENO5, SSP-RK3, per-member CFL, in the FP32 + FP64-refinement
form; the same run times the plain FP64 form on the same members and reports
the speed-up and the relative L2 difference of the vorticity between the two
forms. Other workloads: rsw512 (rotating shallow water channel), eulerpsi256,
eulerpsi512, qg1024/qg4096, euler512, boussinesq512, qgrsw512 (and 1024^2
profiling sizes), each also with a _fp32 suffix; adjoint512 (the discrete
adjoint's cost and finite-difference check). Inputs are seeded synthetic
fields of those configurations' shapes; no dataset is involved. Before the
warm-up the multigrid autotuner picks the solver's schedule (reported as
config.schedule; --no-autotune keeps the default).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--workload rsw512|eulerpsi256|qg4096|...] [--no-autotune]
                  [--no-cpu-baseline] [--no-fp64-form]

--impl gb300 (default): device-timed steps with L2 flushed between steps
(`value`), end-to-end steps through the C ABI with the prognostic state
copied from/to pinned host memory every step (`e2e`; the ensemble reports
the median of three host-timed trials), the dominant kernel
timed alone for the roofline, and the CPU oracle timed on a bounded sample.
--impl reference: the reference algorithm's CPU implementation timed on the
host cores (the oracle port: C sweeps threaded over all cores + numpy
operators + SuperLU), on the same workload.
Under torchrun (N > 1) every rank advances its own replica (no collective on
the data path); the throughput is summed over ranks and timed by the slowest.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (model, builder kwargs, description)
    "rsw512": ("rsw", dict(n=512, seed=0, nislands=3),
               "rsw 512x512 x-periodic channel, 3 islands, f=g=H=1, WENO5, "
               "SSP-RK3, FP64"),
    "eulerpsi256": ("eulerpsi", dict(n=256, seed=0),
                    "eulerpsi 256x256 closed basin, 8 Gaussian vortices, "
                    "WENO5, SSP-RK3, cfl 0.8, FP64, MG-PCG vertex Poisson"),
    "eulerpsi512": ("eulerpsi", dict(n=512, seed=0),
                    "eulerpsi 512x512 closed basin, 8 Gaussian vortices, FP64"),
    "qg4096": ("qg", dict(n=4096, seed=0, nislands=20),
               "qg 4096x4096 basin, 20 islands, Rd=0.02, beta=1, FP64, "
               "MG-PCG Helmholtz"),
    "qg1024": ("qg", dict(n=1024, seed=0, nislands=20),
               "qg 1024x1024 basin, 20 islands, Rd=0.02, beta=1, FP64"),
    "euler512": ("euler", dict(n=512, seed=0, nislands=3),
                 "euler (momentum-pressure) 512x512 closed basin, 3 islands, WENO5 "
                 "vortex force, SSP-RK3, cfl 0.5, FP64, Neumann multigrid-PCG "
                 "pressure projection"),
    "boussinesq512": ("boussinesq", dict(n=512, seed=0, nislands=3),
                      "boussinesq (momentum-pressure + buoyancy) 512x512 closed "
                      "basin, 3 islands, stratification + 2 bubbles, WENO5, "
                      "SSP-RK3, cfl 0.5, FP64, Neumann multigrid-PCG pressure "
                      "projection"),
    "qgrsw512": ("qgrsw", dict(n=512, seed=0, nislands=3, xperiodic=False, f0=10.0),
                 "qgrsw 512x512 closed basin, 3 islands, f0=10, g=H=1, WENO5, "
                 "SSP-RK3, cfl 0.5, FP64, RSW tendency projected on the QG "
                 "manifold by an MG-PCG Helmholtz solve every stage; initial "
                 "state = qg_projection of a thickness bump"),
    "euler1024": ("euler", dict(n=1024, seed=0, nislands=3),
                  "euler 1024x1024 closed basin, 3 islands, FP64 (profiling size: "
                  "working set above the L2)"),
    "boussinesq1024": ("boussinesq", dict(n=1024, seed=0, nislands=3),
                       "boussinesq 1024x1024 closed basin, 3 islands, FP64 (profiling "
                       "size)"),
    "qgrsw1024": ("qgrsw", dict(n=1024, seed=0, nislands=3, xperiodic=False, f0=10.0),
                  "qgrsw 1024x1024 closed basin, 3 islands, f0=10, FP64 (profiling "
                  "size)"),
    "rsw1024": ("rsw", dict(n=1024, seed=0, nislands=3),
                "rsw 1024x1024 x-periodic channel, 3 islands, FP64 (profiling "
                "size: working set above the L2)"),
}

L2_BYTES = 126 * 2 ** 20


ENSEMBLE_DESC = ("ensemble of 256 eulerpsi closed basins, sizes uniform in "
                 "{64,128,192,256,384,512}^2, 0-4 islands each, 8 Gaussian "
                 "vortices, WENO5, SSP-RK3, per-member CFL 0.8")


def solver_roofline(timer, pipelined, handle, workload, peak, peak_src):
    """Roofline of the solver's largest kernel (the level-0 down leg of the
    V-cycle, k_mgp_down when the solver runs the pipelined FP32 kernels, else
    k_mg_down: b and mask read, the pre-smoothed x written, the restricted
    right-hand side written at a quarter of the nodes = (2.25 es + 1) bytes
    per level-0 node), timed alone with CUDA events, L2 flushed."""
    import ctypes
    avg = ctypes.c_double()
    nodes = ctypes.c_int64()
    es = ctypes.c_int()
    rc = timer(handle, 10, 1, ctypes.byref(avg), ctypes.byref(nodes), ctypes.byref(es))
    if rc != 0:
        return None
    pipe = ctypes.c_int()
    if pipelined(handle, ctypes.byref(pipe)) != 0:
        return None
    alg = nodes.value * (2.25 * es.value + 1)
    achieved = alg / (avg.value * 1e-3) / 1e9
    kname = "k_mgp_down" if pipe.value else "k_mg_down"
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak,
            "traffic": read_profile_traffic(f"{kname}_{workload}"),
            "kernel": kname + " (level 0)", "kernel_ms": avg.value,
            "alg_bytes_per_launch": alg, "peak_source": peak_src,
            "binding_roof_ncu": read_profile_text(f"{kname}_{workload}", "binding")}


def max_over_ranks(x, world):
    """The maximum of a per-rank number over the process group (the timing
    rule: the slowest replica's time); the number itself for one process.
    The reduction tensor lives on the backend's device (CUDA for NCCL, the
    host for gloo)."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def replica_value(cells, steps, ms, world):
    """Whole-job cell-updates/s of `world` replicas that each advanced
    `cells` cells `steps` times, timed by the slowest (ms)."""
    return world * cells * steps / (ms / 1e3)


def is_ensemble(name):
    return name.startswith("ensemble")


def precision_of(name):
    return "fp32" if name.endswith("_fp32") else "fp64"


def build_case(name, n=None):
    """The workload's model, seeded synthetic case and description; n: the
    same generator at another grid size."""
    from fluids2d_gb300 import workloads as wl
    base = name[:-5] if name.endswith("_fp32") else name
    model, kw, desc = WORKLOADS[base]
    if n is not None:
        kw = dict(kw, n=n)
    if name.endswith("_fp32"):
        desc = desc.replace("FP64", "FP32 stencils + FP32 multigrid, FP64 CG")
    if model == "rsw":
        case = wl.rsw_case(**kw)
    elif model == "qgrsw":
        case = wl.rsw_case(**kw)
        z = np.zeros_like(case["fields"]["h"])
        case["model"] = "qgrsw"
        case["fields"] = {"u.x": z, "u.y": z.copy(), "h": case["fields"]["h"]}
    elif model == "euler":
        case = wl.euler_case(**kw)
    elif model == "boussinesq":
        case = wl.boussinesq_case(**kw)
    elif model == "eulerpsi":
        case = wl.eulerpsi_case(**kw)
    else:
        case = wl.qg_case(**kw)
    return model, case, desc


def make_gpu_model(model, case, stream_ptr, precision="fp64", tol=None):
    import fluids2d_gb300 as f2d
    from fluids2d_gb300._lib import check, lib
    p = f2d.Param()
    p.model = model
    p.nx, p.ny = case["nx"], case["ny"]
    p.Lx, p.Ly = case["Lx"], case["Ly"]
    p.xperiodic = case.get("xperiodic", False)
    for k in ("f0", "g", "H", "beta"):
        if k in case:
            setattr(p, k, case[k])
    if model == "eulerpsi":
        p.cfl = 0.8
    if model in ("euler", "boussinesq", "qgrsw"):
        p.cfl = 0.5
    p.tend = 1e300
    p.maxite = 10 ** 12
    p.precision = precision
    if tol is not None:
        p.poisson_tol = tol
    m = f2d.Model(p)
    check(lib().f2d_model_set_stream(m._h, stream_ptr))
    m.mesh.msk[:] = case["msk"]
    m.mesh.finalize()
    if "f" in case:
        m.mesh.f = case["f"]
    s = m.state
    for k, v in case["fields"].items():
        if "." in k:
            getattr(getattr(s, k.split(".")[0]), k.split(".")[1])[:] = v
        else:
            getattr(s, k)[:] = v
    if model == "qgrsw":
        m.qg_projection()  # the initial state on the QG manifold
    m.integrator.diag(m.state)
    return m


def prognostic_names(model):
    return {"rsw": ["u.x", "u.y", "h"], "eulerpsi": ["omega"],
            "qg": ["pv"], "euler": ["u.x", "u.y"],
            "boussinesq": ["b", "u.x", "u.y"], "qgrsw": ["u.x", "u.y", "h"]}[model]


# algorithmic bytes per array point of the stage-2 launch of the fused stage
# kernel (FP64): distinct arrays read + written once each
STAGE2_BYTES = {
    # rsw: read u.x,u.y,h,U.x,U.y,ke,p,omega + 3 ds1 (11 x 8) + code (4);
    #      write u.x,u.y,h + 3 ds2 (6 x 8)
    "rsw": 11 * 8 + 4 + 6 * 8,
    # euler (momentum kernel without the mass equation): read u.x, u.y, U.x,
    # U.y, ke, omega + 2 ds1 (8 x 8) + code; write u.x, u.y + 2 ds2 (4 x 8)
    "euler": 8 * 8 + 4 + 4 * 8,
    # boussinesq: euler + b and its ds1 read, b and its ds2 written
    "boussinesq": 10 * 8 + 4 + 6 * 8,
    # qgrsw (momentum kernel in tendency mode): read h, omega, U.x, U.y
    # (4 x 8) + code; write the raw du.x, du.y, dh (3 x 8)
    "qgrsw": 4 * 8 + 4 + 3 * 8,
    # flux form: read q,U.x,U.y,ds1 (4 x 8) + code (4); write q, ds2 (2 x 8)
    "eulerpsi": 4 * 8 + 4 + 2 * 8,
    "qg": 4 * 8 + 4 + 2 * 8,
}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, n in enumerate(names):
                if r[4 + k].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def read_profile_traffic(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", f"{kernel}.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def read_profile_value(kernel, key):
    path = os.path.join(ROOT, "profiles", f"{kernel}.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def read_profile_text(kernel, key):
    """The text after `key:` in the committed ncu summary of `kernel`."""
    path = os.path.join(ROOT, "profiles", f"{kernel}.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith(key + ":"):
            return line.split(":", 1)[1].strip()
    return None


def cpu_oracle_rate(model, case, budget_s, max_steps=None, warmup=1):
    """Oracle port (C sweeps on all host threads + numpy + SuperLU)."""
    from oracle import oracle as O
    p = O.Param(model=model, nx=case["nx"], ny=case["ny"],
                xperiodic=case.get("xperiodic", False), Lx=case["Lx"],
                Ly=case["Ly"], tend=1e300, maxite=10 ** 12)
    for k in ("f0", "g", "H", "beta"):
        if k in case:
            setattr(p, k, case[k])
    if model == "eulerpsi":
        p.cfl = 0.8
    if model in ("euler", "boussinesq", "qgrsw"):
        p.cfl = 0.5
    om = O.Model(p, msk=case["msk"], pysq=False)
    if "f" in case:
        om.mesh.f = case["f"].copy()
    for k, v in case["fields"].items():
        om.s[k][:] = v
    if model == "qgrsw":
        s = om.s
        O.qg_projection(om.mesh, s["u.x"], s["u.y"], s["h"], s["pv"], s["psi"])
    om.diag()
    om.run_steps(warmup)
    n = 0
    t0 = time.perf_counter()
    while True:
        om.run_steps(1)
        n += 1
        el = time.perf_counter() - t0
        if el >= budget_s or (max_steps and n >= max_steps):
            break
    cells = case["nx"] * case["ny"]
    return cells * n / el, n, el, O.num_threads()


def ensemble_cpu_rate(budget_s, steps=1, warmup=1):
    """Oracle port on a stratified sample of the ensemble workload: members
    taken in turn from each grid size (64 .. 512), in draw order, until one
    model step of the sample takes budget_s/steps seconds (measured during
    the first warm-up step, which also builds the models and factorises their
    Poisson matrices), at least one member of every size. Then `steps` timed
    steps, each one model step of every sampled member, timed per member. The
    step time of the whole ensemble is estimated as the sum over sizes of
    (members of that size) x (mean sampled member step time of that size).
    Returns (rate over all members' cells, sample description dict, seconds
    timed, threads, per-step estimated whole-ensemble seconds)."""
    from fluids2d_gb300 import workloads as wl
    from oracle import oracle as O
    members = wl.ensemble_case()
    sizes = sorted({c["nx"] for c in members})
    queues = {n: [c for c in members if c["nx"] == n] for n in sizes}
    count = {n: len(queues[n]) for n in sizes}
    per_step = budget_s / max(1, steps)
    models, el = [], 0.0
    taken = {n: 0 for n in sizes}
    while any(taken[n] < count[n] for n in sizes):
        for n in sizes:
            if taken[n] >= count[n]:
                continue
            c = queues[n][taken[n]]
            taken[n] += 1
            p = O.Param(model="eulerpsi", nx=c["nx"], ny=c["ny"], cfl=0.8, tend=1e300,
                        maxite=10 ** 12)
            om = O.Model(p, msk=c["msk"], pysq=False)
            om.s["omega"][:] = c["fields"]["omega"]
            om.diag()
            t0 = time.perf_counter()
            om.run_steps(1)
            el += time.perf_counter() - t0
            models.append((n, om))
        if el >= per_step:
            break
    for _ in range(max(0, warmup - 1)):
        for _, om in models:
            om.run_steps(1)
    per_member = {n: [] for n in sizes}
    timed = 0.0
    est_steps = []
    for _ in range(max(1, steps)):
        step_t = {n: [] for n in sizes}
        for n, om in models:
            t0 = time.perf_counter()
            om.run_steps(1)
            dt = time.perf_counter() - t0
            step_t[n].append(dt)
            timed += dt
        est_steps.append(sum(count[n] * (sum(step_t[n]) / len(step_t[n])) for n in sizes))
        for n in sizes:
            per_member[n].extend(step_t[n])
    cells_all = sum(c["nx"] * c["ny"] for c in members)
    est = sum(est_steps) / len(est_steps)
    sample = {"members_sampled": {str(n): taken[n] for n in sizes},
              "members_per_size": {str(n): count[n] for n in sizes},
              "ms_per_member_step": {str(n): 1e3 * sum(per_member[n]) / len(per_member[n])
                                     for n in sizes}}
    return cells_all / est, sample, timed, O.num_threads(), est_steps


def reference_as_shipped():
    """The unmodified reference's own timing on the ensemble's grid sizes
    (pure-Python kernels on one core, numba being absent), measured by
    oracle/time_reference.py where the reference's source is available (it
    cannot run on the GPU host); None when that measurement is absent."""
    path = os.path.join(ROOT, "oracle", "reference_timing.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    d["note"] = ("measured with oracle/time_reference.py on the host named here, "
                 "not on this run's host: the reference cannot be installed on the "
                 "GPU host")
    return d


def run_reference(args, rank, world):
    """--impl reference: the CPU implementation of the path on host cores."""
    if is_ensemble(args.workload):
        from fluids2d_gb300 import workloads as wl
        budget = float(os.environ.get("F2D_REF_BUDGET_S", "60"))
        rate, smp, el, cores, est = ensemble_cpu_rate(budget, args.steps, args.warmup)
        members = wl.ensemble_case()
        cells = sum(c["nx"] * c["ny"] for c in members)
        nsamp = sum(smp["members_sampled"].values())
        line = {
            "metric": "cell-updates/s", "value": rate, "unit": "cell-updates/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": len(est),
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(est) / len(est),
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": args.workload, "desc": ENSEMBLE_DESC,
                       "members": len(members), "cells": cells},
            "cpu_baseline": {
                "value": rate, "unit": "cell-updates/s", "cores": cores,
                "kind": "port",
                "sample": f"stratified: {nsamp} of the {len(members)} members "
                          f"({smp['members_sampled']} by grid size), one model step of "
                          f"each per timed step, {len(est)} timed steps, {el:.1f} s on "
                          f"{cores} host threads (set-up and SuperLU factorisation in "
                          f"the warm-up, untimed); ms_per_step is the whole-ensemble "
                          f"step time estimated as the sum over sizes of members x "
                          f"mean member step time",
                "per_size": smp},
            "e2e": {"value": rate, "unit": "cell-updates/s",
                    "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        ref = reference_as_shipped()
        if ref:
            line["cpu_baseline"]["reference_as_shipped"] = ref
        print(json.dumps(line), flush=True)
        return
    model, case, desc = build_case(args.workload)
    what = args.workload
    if case["nx"] * case["ny"] > 1024 * 1024:
        # SuperLU cannot factorise the full grid in the host's memory: the
        # same generator at 1024^2, rate per cell update
        case = build_case(args.workload, n=1024)[1]
        what = f"{args.workload}'s generator at 1024x1024 (same seed and islands)"
    budget = float(os.environ.get("F2D_REF_BUDGET_S", "60"))
    rate, n, el, cores = cpu_oracle_rate(model, case, budget,
                                         max_steps=args.steps,
                                         warmup=min(args.warmup, 1))
    line = {
        "metric": "cell-updates/s", "value": rate, "unit": "cell-updates/s",
        "impl": "reference", "n_gpus": args.gpus, "steps": n,
        "warmup": args.warmup, "ms_per_step": 1e3 * el / n,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "desc": desc},
        "cpu_baseline": {
            "value": rate, "unit": "cell-updates/s", "cores": cores,
            "kind": "port",
            "sample": f"{n} model steps (of the requested {args.steps}) of "
                      f"{what} on {cores} host threads, "
                      f"{el:.1f} s, after {min(args.warmup, 1)} warm-up"},
        "e2e": {"value": rate, "unit": "cell-updates/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _ensemble_make(prec, members, stream):
    import fluids2d_gb300 as f2d
    p = f2d.Param()
    p.model = "eulerpsi"
    p.cfl = 0.8
    p.tend = 1e300
    p.maxite = 10 ** 12
    p.precision = prec
    e = f2d.Ensemble(p, [(c["nx"], c["ny"]) for c in members],
                     [c["msk"] for c in members])
    e.set_stream(stream.cuda_stream)
    for b, c in enumerate(members):
        e.set_field(b, "omega", c["fields"]["omega"])
    e.diag()
    return e


def _ensemble_time(e, steps, warmup, stream, flush, dev, world):
    import torch
    from fluids2d_gb300._lib import check, lib
    L = lib()
    for _ in range(warmup):
        check(L.f2d_ensemble_run(e._h, 1))
    e.sync()
    st0 = e.stats()
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        for k in range(steps):
            flush.zero_()
            ev0[k].record(stream)
            check(L.f2d_ensemble_run(e._h, 1))
            ev1[k].record(stream)
        torch.cuda.synchronize()
    e.sync()
    ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in zip(ev0, ev1)), world)
    st = e.stats()
    return ms, st0, st, clk.summary()


def plain_fp64_ms_per_step(members, stream, flush, steps=3, warmup=2, stride=4):
    """Time of one ensemble step in the plain FP64 form: every member as its
    own single FP64 model, advanced one after another (no batching). Times a
    systematic sample (every `stride`-th member; the members are independent
    draws) with CUDA events and scales the summed per-step time to all
    members. Returns (ms per ensemble step, members timed)."""
    import ctypes
    import torch
    from fluids2d_gb300._lib import check, lib
    L = lib()
    sample = members[::stride]
    tot = 0.0
    for c in sample:
        m = make_gpu_model("eulerpsi", c, ctypes.c_void_p(stream.cuda_stream), "fp64")
        for _ in range(warmup):
            check(L.f2d_run(m._h, 1))
        check(L.f2d_sync(m._h))
        ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        for k in range(steps):
            flush.zero_()
            ev0[k].record(stream)
            check(L.f2d_run(m._h, 1))
            ev1[k].record(stream)
        torch.cuda.synchronize()
        tot += sum(a.elapsed_time(b) for a, b in zip(ev0, ev1)) / steps
        del m
    return tot * len(members) / len(sample), len(sample)


def run_gpu_ensemble(args, rank, world):
    import ctypes
    import torch
    from fluids2d_gb300 import workloads as wl
    from fluids2d_gb300._lib import check, lib
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    prec = precision_of(args.workload)
    members = wl.ensemble_case(seed=rank)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    e = _ensemble_make(prec, members, stream)
    # the multigrid schedule picked by the autotuner (outside the timed region)
    tune = None if args.no_autotune else e.autotune(reps=2)
    L = lib()
    h = e._h
    cells = sum(c["nx"] * c["ny"] for c in members)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    ms, st0, st, clocks = _ensemble_time(e, args.steps, args.warmup, stream, flush,
                                         dev, world)
    pcg_iters = st["poisson_iters"] - st0["poisson_iters"]
    loops = st["loop_iters"] - st0["loop_iters"]
    value = replica_value(cells, args.steps, ms, world)
    # the plain FP64 form on the same members and step count, for the
    # speed-up and the difference between the forms
    fp64_form = None
    if prec == "fp32" and not args.no_fp64_form:
        e64 = _ensemble_make("fp64", members, stream)
        tune64 = None if args.no_autotune else e64.autotune(reps=2)
        ms64, _, _, _ = _ensemble_time(e64, args.steps, args.warmup, stream, flush,
                                       dev, world)
        num = den = 0.0
        for b in range(len(members)):
            a32 = e.get_field(b, "omega")
            a64 = e64.get_field(b, "omega")
            num += float(np.sum((a32 - a64) ** 2))
            den += float(np.sum(a64 ** 2))
        fp64_form = {"value": world * cells * args.steps / (ms64 / 1e3),
                     "ms_per_step": ms64 / args.steps, "schedule": tune64,
                     "speedup_fp32_refine_vs_fp64": ms64 / ms,
                     "omega_rel_l2_fp32_vs_fp64": (num / den) ** 0.5,
                     "steps": args.warmup + args.steps}
        del e64
        pms, nsamp = plain_fp64_ms_per_step(members, stream, flush)
        fp64_form["plain_fp64_per_member"] = {
            "value": world * cells / (pms / 1e3), "ms_per_step": pms,
            "speedup_fp32_refine_batched_vs_plain_fp64": pms / (ms / args.steps),
            "sample": f"{nsamp} of {len(members)} members (every 4th), each a "
                      "single FP64 model, 2 warm-up + 3 timed steps, summed "
                      "per-step times scaled to all members"}
    # end to end: every member's vorticity from pinned host memory and back
    # (all members' vorticity in one pinned buffer, one copy each way per step)
    host = torch.empty(e.packed_size(), dtype=torch.float64, pin_memory=True)
    hp = ctypes.c_void_p(host.data_ptr())
    check(L.f2d_ensemble_fields_get(h, b"omega", hp, 0))
    e2e_steps = max(1, min(args.steps, 20))
    # three trials of e2e_steps steps each (host clock around the loop), the
    # median reported: one short host-timed window is exposed to host jitter
    trials = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            check(L.f2d_ensemble_fields_set(h, b"omega", hp, 1))
            check(L.f2d_ensemble_run(h, 1))
            check(L.f2d_ensemble_fields_get(h, b"omega", hp, 1))
        e.sync()
        trials.append(world * cells * e2e_steps / (time.perf_counter() - t0))
    io = sum((c["ny"] + 6) * (c["nx"] + 6) * 8 for c in members)
    e2e = float(np.median(trials))
    # roofline: the batched flux-form stage kernel of all members
    avg = ctypes.c_double()
    check(L.f2d_ensemble_time_stage(h, 2, 10, 1, ctypes.byref(avg)))
    npts = sum((c["ny"] + 6) * (c["nx"] + 6) for c in members)
    per = STAGE2_BYTES["eulerpsi"]
    if prec == "fp32":
        per = (per - 4) // 2 + 4
    alg_bytes = per * npts
    achieved = alg_bytes / (avg.value * 1e-3) / 1e9
    try:
        peak, peak_src = float(json.load(open(os.path.join(
            ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]), "measured"
    except Exception:
        peak, peak_src = 6800.0, "fallback"
    kname = "k_ens_fluxform_stage"
    line = {
        "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if prec == "fp32" else "f64", "data": "synthetic",
        "config": {"workload": args.workload, "desc": ENSEMBLE_DESC,
                   "members": len(members), "cells": cells,
                   "precision": ("FP32 stencils + FP32 multigrid inner CG, FP64 "
                                 "iterative refinement (Poisson solution at FP64 "
                                 "accuracy, tol 1e-12)" if prec == "fp32"
                                 else "FP64 throughout"),
                   "l2": "flushed between timed steps (256 MB write)",
                   "schedule": tune,
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e, "unit": "cell-updates/s",
                "h2d_bytes_per_step": io, "d2h_bytes_per_step": io,
                "steps": e2e_steps, "trials": trials,
                "reported": "median of 3 trials"},
        "roofline": solver_roofline(L.f2d_ensemble_time_solver,
                                    L.f2d_ensemble_solver_pipelined, h, args.workload,
                                    peak, peak_src),
        "roofline_stage": {"bound": "hbm", "achieved": achieved, "peak": peak,
                           "unit": "GB/s", "frac": achieved / peak,
                           "traffic": read_profile_traffic(f"{kname}_{args.workload}"),
                           "kernel": kname, "kernel_ms": avg.value,
                           "alg_bytes_per_launch": alg_bytes, "peak_source": peak_src},
        "gpu_launches": st["launches_per_step"] * args.steps
                        + st["launches_per_iter"] * loops,
        "poisson_iters_sum_over_members": pcg_iters,
        "cg_loop_iters": loops,
        "solver_per_solve": {
            # 3 solves per member and step (one per RK3 stage diagnostic)
            "pcg_iters_per_member": pcg_iters / (3 * args.steps * len(members)),
            "refine_rounds_per_member": (st["refine_rounds"] - st0["refine_rounds"])
                                        / (3 * args.steps * len(members)),
            "loop_iters": loops / (3 * args.steps)},
        "clocks": clocks,
    }
    if fp64_form:
        line["fp64_form"] = fp64_form
    if rank == 0 and not args.no_cpu_baseline:
        budget = float(os.environ.get("F2D_CPU_BUDGET_S", "15"))
        rate, smp, el, cores, _ = ensemble_cpu_rate(budget, 1, 1)
        line["cpu_baseline"] = {
            "value": rate, "unit": "cell-updates/s", "cores": cores, "kind": "port",
            "sample": f"stratified: {sum(smp['members_sampled'].values())} members "
                      f"({smp['members_sampled']} by grid size), one model step of each "
                      f"after a warm-up step, {el:.1f} s on {cores} host threads; the "
                      f"whole-ensemble step time estimated as the sum over sizes of "
                      f"members x mean member step time",
            "per_size": smp}
        ref = reference_as_shipped()
        if ref:
            line["cpu_baseline"]["reference_as_shipped"] = ref
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_gpu_adjoint(args, rank, world):
    """Differentiation workload: eulerpsi 512x512 closed basin, loss = final
    enstrophy + L2 misfit to a seeded target after 400 fixed-dt steps,
    gradient w.r.t. the initial vorticity through the adjoint kernels with
    checkpoints every 20 steps; FP32 forward (FP64-refined Poisson) by
    default. Reports the gradient throughput, the cost of forward+backward
    relative to a plain forward of the same steps, the FP32 gradient against
    the FP64 one, and the FP64 gradient against central finite differences
    along random directions."""
    import ctypes
    import torch
    from fluids2d_gb300 import workloads as wl
    from fluids2d_gb300.adjoint import rollout
    from fluids2d_gb300._lib import check, lib
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    n = int(os.environ.get("F2D_ADJ_N", "512"))
    nsteps = int(os.environ.get("F2D_ADJ_STEPS", "400"))
    every = 20
    prec = "fp64" if args.workload.endswith("_fp64") else "fp32"
    case = wl.eulerpsi_case(n=n, seed=rank)
    rng = np.random.default_rng(1000 + rank)
    target_np = wl.band_limited_field(n, n, 2, 8, seed=2000 + rank) * case["fields"][
        "omega"].std() * case["msk"]
    area = (1.0 / n) ** 2
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    def model(precision, tol=None):
        return make_gpu_model("eulerpsi", case, ctypes.c_void_p(stream.cuda_stream),
                              precision, tol)

    m = model(prec)
    m.set_dt()
    dt = m.time.dt  # the CFL step of the initial state, then held fixed
    target = torch.tensor(target_np, device="cuda")
    w0 = torch.tensor(case["fields"]["omega"], device="cuda")

    def loss_fn(w):
        return (0.5 * (w ** 2).mean() + ((w - target) ** 2).mean()) / area ** 2

    def timed(fn):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        out = fn()
        b.record(stream)
        torch.cuda.synchronize()
        return out, a.elapsed_time(b)

    # plain forward of the same steps (no checkpoints), graph-captured steps
    L = lib()
    for _ in range(args.warmup):
        check(L.f2d_step(m._h, 1))
    check(L.f2d_sync(m._h))
    _, ms_plain = timed(lambda: (check(L.f2d_step(m._h, nsteps)), check(L.f2d_sync(m._h))))
    # warm-up of the differentiable path (graph captures), then timed
    x = w0.clone().requires_grad_(True)
    g = torch.autograd.grad(loss_fn(rollout(m, x, min(nsteps, 2 * every), dt, every)), x)
    x = w0.clone().requires_grad_(True)
    wT, ms_fwd = timed(lambda: rollout(m, x, nsteps, dt, every))
    lo = loss_fn(wT)
    (g,), ms_bwd = timed(lambda: torch.autograd.grad(lo, x))
    cells = n * n
    # FP64 gradient for the precision comparison and the finite differences
    m64 = model("fp64", tol=1e-14)
    x64 = w0.clone().requires_grad_(True)
    (g64,) = torch.autograd.grad(loss_fn(rollout(m64, x64, nsteps, dt, every)), x64)
    fluid = torch.tensor(case["msk"] > 0, device="cuda")
    ndir = int(os.environ.get("F2D_ADJ_FD_DIRS", "16"))
    errs = []
    with torch.no_grad():
        for k in range(ndir):
            v = torch.tensor(rng.standard_normal(w0.shape), device="cuda") * fluid
            h = 1e-7 * float(w0.abs().max()) / float(v.abs().max())
            fp = loss_fn(rollout(m64, w0 + h * v, nsteps, dt, every))
            fm = loss_fn(rollout(m64, w0 - h * v, nsteps, dt, every))
            fd = float(fp - fm) / (2 * h)
            an = float((g64 * v).sum())
            errs.append(abs(fd - an) / abs(an))
    gdiff = float(torch.linalg.norm(g - g64) / torch.linalg.norm(g64))
    value = world * cells * nsteps / ((ms_fwd + ms_bwd) / 1e3)
    line = {
        "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s",
        "n_gpus": world, "steps": nsteps, "warmup": args.warmup,
        "ms_per_step": (ms_fwd + ms_bwd) / nsteps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if prec == "fp32" else "f64", "data": "synthetic",
        "config": {"workload": args.workload,
                   "desc": f"gradient of final enstrophy + L2 misfit to a seeded "
                           f"target after {nsteps} fixed-dt RK3 steps of eulerpsi "
                           f"{n}x{n} closed basin w.r.t. the initial vorticity; "
                           f"adjoint WENO5/RK3/Poisson kernels, checkpoints every "
                           f"{every} steps",
                   "precision": prec, "parallelism": f"replicas x{world}"},
        "adjoint": {
            "ms_forward_plain": ms_plain, "ms_forward_checkpointed": ms_fwd,
            "ms_backward": ms_bwd,
            "cost_forward_plus_backward_over_forward": (ms_fwd + ms_bwd) / ms_plain,
            "cost_backward_over_forward": ms_bwd / ms_plain,
            "grad_rel_l2_vs_fp64_gradient": gdiff,
            "fd_directions": ndir,
            "fd_rel_err_max": max(errs) if errs else None,
            "fd_rel_err_median": float(np.median(errs)) if errs else None,
            "fd_setup": "FP64 forward, Poisson tol 1e-14, central differences, "
                        "step 1e-7 max|omega0|, random directions on fluid cells"},
        "gpu_launches": None,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_gpu(args, rank, world):
    if args.workload.startswith("adjoint"):
        return run_gpu_adjoint(args, rank, world)
    if is_ensemble(args.workload):
        return run_gpu_ensemble(args, rank, world)
    import torch
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    from fluids2d_gb300._lib import check, lib
    import ctypes

    model, case, desc = build_case(args.workload)
    # one non-default stream for the model, the L2 flushes and the events
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    assert stream.cuda_stream != 0
    prec = precision_of(args.workload)
    m = make_gpu_model(model, case, ctypes.c_void_p(stream.cuda_stream), prec)
    # the multigrid schedule picked by the autotuner (outside the timed region)
    tune = (m.autotune(reps=2) if not args.no_autotune
            and model in ("eulerpsi", "qg", "qgrsw") else None)
    h = m._h
    L = lib()
    cells = case["nx"] * case["ny"]
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")

    # warm-up (graph capture happens here)
    for _ in range(args.warmup):
        check(L.f2d_run(h, 1))
    check(L.f2d_sync(h))
    it0 = m.poisson_iterations()

    # ---- device-timed steps, L2 flushed between steps ----------------------
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        for k in range(args.steps):
            flush.zero_()
            ev0[k].record(stream)
            check(L.f2d_run(h, 1))
            ev1[k].record(stream)
        torch.cuda.synchronize()
    check(L.f2d_sync(h))
    ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in zip(ev0, ev1)), world)
    pcg_iters = m.poisson_iterations() - it0
    value = replica_value(cells, args.steps, ms, world)

    # ---- end to end through the C ABI with pinned host state ---------------
    names = prognostic_names(model)
    host = {}
    for n in names:
        t = torch.empty((case["ny"] + 6, case["nx"] + 6), dtype=torch.float64,
                        pin_memory=True)
        host[n] = t
        check(L.f2d_field_get(h, n.encode(), ctypes.c_void_p(t.data_ptr())))
    e2e_steps = max(1, min(args.steps, 200))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for n in names:
            check(L.f2d_field_set_async(h, n.encode(),
                                        ctypes.c_void_p(host[n].data_ptr())))
        check(L.f2d_run(h, 1))
        for n in names:
            check(L.f2d_field_get_async(h, n.encode(),
                                        ctypes.c_void_p(host[n].data_ptr())))
    check(L.f2d_sync(h))
    e2e_s = time.perf_counter() - t0
    bytes_io = len(names) * (case["ny"] + 6) * (case["nx"] + 6) * 8
    e2e = world * cells * e2e_steps / e2e_s

    # ---- roofline of the dominant kernel: the fused stage kernel -----------
    avg = ctypes.c_double()
    check(L.f2d_time_stage(h, 2, 20, 1, ctypes.byref(avg)))
    npts = (case["ny"] + 6) * (case["nx"] + 6)
    alg_bytes = STAGE2_BYTES[model] * npts
    if prec == "fp32":  # 4-byte fields, the 4-byte code word unchanged
        alg_bytes = ((STAGE2_BYTES[model] - 4) // 2 + 4) * npts
    achieved = alg_bytes / (avg.value * 1e-3) / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        peak, peak_src = float(peaks["hbm_gbs"]), "measured"
    except Exception:
        peak, peak_src = 6800.0, "fallback"
    kname = {"rsw": "k_rsw_stage", "eulerpsi": "k_fluxform_stage",
             "qg": "k_fluxform_stage", "euler": "k_rsw_stage",
             "boussinesq": "k_rsw_stage", "qgrsw": "k_rsw_stage"}[model]
    traffic = read_profile_traffic(f"{kname}_{args.workload}")
    fp64_pct = read_profile_value(f"{kname}_{args.workload}", "fp64_pipe_pct")

    # launches in the timed region: fixed kernels per step + Poisson bodies
    _, nfix, body = m.stats()
    launches = nfix * args.steps + body * pcg_iters

    line = {
        "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if prec == "fp32" else "f64",
        "data": "synthetic",
        "config": {"workload": args.workload, "desc": desc,
                   "grid": [case["ny"], case["nx"]],
                   "l2": "flushed between timed steps (256 MB write)",
                   "schedule": tune,
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e, "unit": "cell-updates/s",
                "h2d_bytes_per_step": bytes_io, "d2h_bytes_per_step": bytes_io,
                "steps": e2e_steps},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": kname,
                     "kernel_ms": avg.value, "alg_bytes_per_launch": alg_bytes,
                     "peak_source": peak_src,
                     "binding_roof_ncu": ({"fp64_pipe_active_pct": fp64_pct}
                                          if fp64_pct is not None else None)},
        "gpu_launches": launches,
        "poisson_iters": pcg_iters,
        "clocks": clk.summary(),
    }
    if model != "rsw":
        # the Poisson solve dominates the step: its largest kernel is the
        # roofline kernel, the fused stage is reported beside it
        sr = solver_roofline(L.f2d_time_solver, L.f2d_solver_pipelined, h, args.workload,
                             peak, peak_src)
        if sr is not None:
            line["roofline_stage"] = line["roofline"]
            line["roofline"] = sr
    if rank == 0 and not args.no_cpu_baseline:
        budget = float(os.environ.get("F2D_CPU_BUDGET_S", "15"))
        cpu_case, what = case, args.workload
        if case["nx"] * case["ny"] > 1024 * 1024:
            # SuperLU's factorisation of the full grid does not fit the host's
            # memory: the same generator at 1024^2, rate per cell update
            cpu_case = build_case(args.workload, n=1024)[1]
            what = f"{args.workload}'s generator at 1024x1024 (same seed and islands)"
        rate, n, el, cores = cpu_oracle_rate(model, cpu_case, budget)
        line["cpu_baseline"] = {
            "value": rate, "unit": "cell-updates/s", "cores": cores,
            "kind": "port",
            "sample": f"{n} model steps of {what} after 1 warm-up, "
                      f"{el:.1f} s on {cores} host threads"}
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="ensemble256_fp32",
                    choices=sorted(WORKLOADS) + sorted(k + "_fp32" for k in WORKLOADS)
                    + ["ensemble256", "ensemble256_fp32", "adjoint512",
                       "adjoint512_fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-form", action="store_true",
                    help="ensemble FP32 workload: skip the plain-FP64 comparison")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default multigrid schedule (no autotuner pass "
                         "before the warm-up)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    run_gpu(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
