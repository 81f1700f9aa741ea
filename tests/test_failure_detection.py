"""Failure detection on the GPU, in forms that fault and hang nothing.

* A NaN planted on the host in an initial state: the Poisson solve's
  residual and the CFL time step become NaN (as numpy's max and Python's min
  make the reference's set_dt NaN, model.py:83-87), the device records the
  non-finite status and f2d_sync / f2d_ensemble_sync report it; after a
  finite state is written back, the model steps as the oracle does.
* A TMA tile wait that runs out: the test switch f2d_test_tma_wait makes
  every stage kernel, after its tile has landed, wait for a barrier phase
  that nothing completes, with a 10 ms limit. The kernel records the time-out
  and returns; f2d_sync reports it; with the switch off the same model steps
  correctly again (the context stays usable).
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import fluids2d_gb300 as f2d  # noqa: E402
from fluids2d_gb300 import workloads as wl  # noqa: E402
from fluids2d_gb300._lib import check, lib  # noqa: E402
from test_gpu_parity import (STEP_TOL, _ensemble, _model, _oracle_like,  # noqa: E402
                             compare)


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.fixture
def tma_wait_switch():
    yield lambda on: check(lib().f2d_test_tma_wait(1 if on else 0, 10.0))
    check(lib().f2d_test_tma_wait(0, 0.0))


def _eulerpsi(case, **kw):
    m = _model("eulerpsi", case["nx"], case["ny"], case["msk"], cfl=0.8, tend=1e300,
               maxite=10 ** 9, **kw)
    m.state.omega[:] = case["fields"]["omega"]
    return m


def _reset_and_check_against_oracle(m, case, kind="eulerpsi", nsteps=2):
    """Write a finite state, step, compare with the oracle."""
    s = m.state
    for name in s._fields:
        v = getattr(s, name)
        if hasattr(v, "_fields"):
            v.x[:] = 0.0
            v.y[:] = 0.0
        else:
            v[:] = 0.0
    for k, v in case["fields"].items():
        if "." in k:
            getattr(getattr(s, k.split(".")[0]), k.split(".")[1])[:] = v
        else:
            getattr(s, k)[:] = v
    m.time.ite = 0
    m.time.t = 0.0
    m.integrator.diag(s)
    om = _oracle_like(case, kind, cfl=m.param.cfl)
    for _ in range(nsteps):
        om.run_steps(1)
        m.advance(1)
        assert abs(m.time.dt - om.dt) <= 1e-10 * om.dt
        compare(m, lambda k: om.s.get(k), STEP_TOL)
    m.sync()


def test_nan_vorticity_reports_nonfinite_then_recovers():
    case = wl.eulerpsi_case(n=64, ny=48, seed=3, nislands=2)
    m = _eulerpsi(case)
    w = case["fields"]["omega"].copy()
    j, i = 20, 30
    assert case["msk"][j, i] == 1
    w[j, i] = np.nan
    m.state.omega[:] = w
    m.integrator.diag(m.state)
    with pytest.raises(f2d.F2DError, match="non-finite"):
        m.sync()
    # the reference's set_dt on the same state: np.max propagates the NaN of
    # U, min(nan, dtmax) keeps it
    om = _oracle_like(dict(case, fields={"omega": w}), "eulerpsi", cfl=0.8)
    om.set_dt()
    assert np.isnan(om.dt)
    m.set_dt()
    assert np.isnan(m.time.dt)
    with pytest.raises(f2d.F2DError, match="non-finite"):
        m.sync()
    m.sync()  # reported once, then cleared
    _reset_and_check_against_oracle(m, case)


def test_nan_member_reports_nonfinite_in_ensemble():
    members = [wl.eulerpsi_case(n=48, ny=40, seed=21, nislands=1),
               wl.eulerpsi_case(n=64, ny=64, seed=22, nislands=2)]
    e = _ensemble(members, "fp64")
    e.sync()
    w = members[1]["fields"]["omega"].copy()
    w[30, 30] = np.nan
    e.set_field(1, "omega", w)
    e.diag()
    with pytest.raises(f2d.F2DError, match="non-finite"):
        e.sync()
    e.run(1)
    with pytest.raises(f2d.F2DError, match="non-finite"):
        e.sync()
    assert np.isnan(e.time(1)[1])  # member 1's dt is NaN ...
    assert np.isfinite(e.time(0)[1])  # ... member 0's is not


@pytest.mark.parametrize("kind", ["eulerpsi", "rsw"])
def test_tma_wait_timeout_reports_then_recovers(kind, tma_wait_switch):
    if kind == "eulerpsi":
        case = wl.eulerpsi_case(n=64, ny=48, seed=3, nislands=2)
        m = _eulerpsi(case)
    else:
        case = wl.rsw_case(n=64, ny=48, seed=4, nislands=2)
        m = _model("rsw", 64, 48, case["msk"], xperiodic=True, f0=case["f0"],
                   g=case["g"], H=case["H"], tend=1e300, maxite=10 ** 9)
        m.state.h[:] = case["fields"]["h"]
    m.integrator.diag(m.state)
    m.sync()
    tma_wait_switch(True)
    m.advance(1)
    with pytest.raises(f2d.F2DError, match="TMA tile load timed out"):
        m.sync()
    tma_wait_switch(False)
    m.sync()
    _reset_and_check_against_oracle(m, case, kind)


def test_tma_wait_timeout_in_ensemble(tma_wait_switch):
    members = [wl.eulerpsi_case(n=48, ny=40, seed=21, nislands=1),
               wl.eulerpsi_case(n=72, ny=64, seed=22, nislands=1)]
    e = _ensemble(members, "fp64")
    e.sync()
    tma_wait_switch(True)
    e.run(1)
    with pytest.raises(f2d.F2DError, match="TMA tile load timed out"):
        e.sync()
    tma_wait_switch(False)
    e2 = _ensemble(members, "fp64")
    e2.run(2)
    e2.sync()
    for b, c in enumerate(members):
        om = _oracle_like(c, "eulerpsi", cfl=0.8)
        om.run_steps(2)
        err = np.linalg.norm(e2.get_field(b, "omega") - om.s["omega"]) / np.linalg.norm(
            om.s["omega"])
        assert err <= STEP_TOL


def test_tma_wait_switch_rejects_bad_limit():
    assert lib().f2d_test_tma_wait(1, 0.0) != 0
    assert lib().f2d_test_tma_wait(1, 5000.0) != 0
    assert b"limit_ms" in lib().f2d_last_error()
    check(lib().f2d_test_tma_wait(0, 0.0))
