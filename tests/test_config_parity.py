"""GPU parity at the sizes of the benchmark configurations, against the
oracle (whose sweeps, operators and SuperLU solves are pinned to the
unmodified reference by tests/test_oracle_golden.py).

* eulerpsi 256^2 closed basin, 8 Gaussian vortices, WENO5, SSP-RK3, CFL 0.8,
  the whole 200-step run (states compared every 10 steps, dt every step);
* rsw 512^2 x-periodic channel with 3 islands, f = g = H = 1, 20 steps;
* the batched ensemble: one member of each grid size 64/128/192/256/384/512
  taken from the benchmark's own 256-member draw (ensemble_case(seed=0)),
  advanced together in one FP64 ensemble for 5 steps, each member against its
  own oracle run;
* qg with 20 islands and the beta-plane at 1024^2 (the reduced size of the
  4096^2 configuration at which SuperLU still factors), 3 steps.

FP64 form: every field within 1e-10 relative L2 of the oracle at every
comparison, dt within 1e-10 relative at every step.

FP32 form (FP32 stencils and multigrid, FP64-refined Poisson solution): the
vorticity / potential vorticity and the streamfunction within 1e-6 relative
L2 of the FP64 oracle after the same steps, for the ensemble members, the
eulerpsi 256^2 configuration and qg 1024^2.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import fluids2d_gb300 as f2d  # noqa: E402
from fluids2d_gb300 import workloads as wl  # noqa: E402
from test_gpu_parity import (STEP_TOL, _ensemble, _model, _oracle_like,  # noqa: E402
                             compare, rel_l2)

FP32_TOL = 1e-6


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _gpu_like(case, kind, **extra):
    kw = dict(xperiodic=case.get("xperiodic", False), Lx=case["Lx"], Ly=case["Ly"],
              tend=1e300, maxite=10 ** 9, **extra)
    for k in ("f0", "g", "H", "beta"):
        if k in case:
            kw[k] = case[k]
    m = _model(kind, case["nx"], case["ny"], case["msk"], **kw)
    if "f" in case:
        m.mesh.f = case["f"]
    s = m.state
    for k, v in case["fields"].items():
        if "." in k:
            getattr(getattr(s, k.split(".")[0]), k.split(".")[1])[:] = v
        else:
            getattr(s, k)[:] = v
    m.integrator.diag(s)
    return m


def _run_pair(kind, case, nsteps, every=1, **extra):
    """Step the oracle and the GPU model side by side; compare every field
    every `every` steps and dt at every step."""
    om = _oracle_like(case, kind, **extra)
    m = _gpu_like(case, kind, **extra)
    compare(m, lambda k: om.s.get(k), STEP_TOL)
    worst = {}
    for n in range(1, nsteps + 1):
        om.run_steps(1)
        m.advance(1)
        assert abs(m.time.dt - om.dt) <= 1e-10 * om.dt, (n, m.time.dt, om.dt)
        if n % every == 0 or n == nsteps:
            w = compare(m, lambda k: om.s.get(k), STEP_TOL)
            for k, e in w.items():
                worst[k] = max(worst.get(k, 0.0), e)
    m.sync()
    print(f"{kind} {case['nx']}x{case['ny']} {nsteps} steps, worst rel L2:",
          {k: f"{v:.1e}" for k, v in worst.items()})
    return m, om


def test_eulerpsi256_config_200_steps():
    case = wl.eulerpsi_case(n=256, seed=0)
    _run_pair("eulerpsi", case, 200, every=10, cfl=0.8)


def test_rsw512_config_channel_islands():
    case = wl.rsw_case(n=512, seed=0, nislands=3)
    m, om = _run_pair("rsw", case, 20, every=5)
    # the run moved the state: the bump radiates gravity waves
    assert np.abs(m.state.u.x).max() > 1e-6


def test_qg1024_islands_beta():
    case = wl.qg_case(n=1024, seed=0, nislands=20)
    _run_pair("qg", case, 3)


def _size_members(count=256, seed=0):
    """One member of each grid size from the benchmark's ensemble draw."""
    members = wl.ensemble_case(count=count, seed=seed)
    pick = {}
    for c in members:
        pick.setdefault(c["nx"], c)
    sizes = sorted(pick)
    assert sizes == [64, 128, 192, 256, 384, 512], sizes
    return [pick[n] for n in sizes]


def _oracle_run(c, nsteps):
    om = _oracle_like(c, "eulerpsi", cfl=0.8)
    states = []
    for _ in range(nsteps):
        om.run_steps(1)
        states.append({k: om.s[k].copy() for k in ("omega", "psi", "U.x", "U.y")})
    return om, states


@pytest.fixture(scope="module")
def size_members_oracle():
    members = _size_members()
    runs = [_oracle_run(c, 5) for c in members]
    return members, runs


def test_ensemble_members_every_size_fp64(size_members_oracle):
    members, runs = size_members_oracle
    e = _ensemble(members, "fp64")
    worst = 0.0
    for n in range(5):
        e.run(1)
        e.sync()
        for b, c in enumerate(members):
            om, states = runs[b]
            t, dt, ite = e.time(b)
            ref = states[n]
            for k in ("omega", "psi", "U.x", "U.y"):
                err = rel_l2(e.get_field(b, k), ref[k])
                worst = max(worst, err)
                assert err <= STEP_TOL, (c["nx"], n + 1, k, err)
    for b, (om, _) in enumerate(runs):
        t, dt, ite = e.time(b)
        assert ite == 5 and abs(dt - om.dt) <= 1e-10 * om.dt
    print(f"FP64 ensemble, sizes 64..512, 5 steps: worst rel L2 {worst:.1e}")


def test_ensemble_members_every_size_fp32(size_members_oracle):
    """The FP32 + FP64-refinement form of the benchmark against the FP64
    oracle: vorticity and streamfunction of every member within 1e-6."""
    members, runs = size_members_oracle
    e = _ensemble(members, "fp32")
    e.run(5)
    e.sync()
    errs = {}
    for b, c in enumerate(members):
        ref = runs[b][1][-1]
        for k in ("omega", "psi"):
            errs[(c["nx"], k)] = rel_l2(e.get_field(b, k), ref[k])
    print("FP32 ensemble vs FP64 oracle after 5 steps:",
          {f"{n}/{k}": f"{v:.1e}" for (n, k), v in errs.items()})
    bad = {k: v for k, v in errs.items() if v > FP32_TOL}
    assert not bad, bad


@pytest.mark.parametrize("kind", ["eulerpsi", "qg"])
def test_fp32_config_vs_fp64_oracle(kind):
    """eulerpsi 256^2 (20 steps) and qg 1024^2 with islands and beta (3
    steps) in the FP32 form: the prognostic field and psi within 1e-6 of the
    FP64 oracle."""
    if kind == "eulerpsi":
        case, nsteps, q = wl.eulerpsi_case(n=256, seed=0), 20, "omega"
    else:
        case, nsteps, q = wl.qg_case(n=1024, seed=0, nislands=20), 3, "pv"
    om = _oracle_like(case, kind, cfl=0.8) if kind == "eulerpsi" else _oracle_like(case, kind)
    extra = dict(cfl=0.8) if kind == "eulerpsi" else {}
    m = _gpu_like(case, kind, precision="fp32", **extra)
    om.run_steps(nsteps)
    m.advance(nsteps)
    m.sync()
    errs = {k: rel_l2(getattr(m.state, k), om.s[k]) for k in (q, "psi")}
    print(f"FP32 {kind} {case['nx']}^2 after {nsteps} steps vs FP64 oracle:",
          {k: f"{v:.1e}" for k, v in errs.items()})
    assert all(v <= FP32_TOL for v in errs.values()), errs
    assert abs(m.time.t - om.t) <= 1e-6 * om.t
