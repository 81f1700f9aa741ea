"""The right-hand-side plug point, single stages, forcing terms and the
classic inner product, on the GPU through the C ABI.

* f2d_rhs (the reference's rhs(s, ds), equations.py:73-157, with tracer and
  forcing terms) against the reference's own rhs evaluation on the initial
  state of every model fixture (``rhs0/<var>``, written by make_golden.py);
* the reference's SSP-RK3 loop (integrators.py:92-107, restated here on host
  numpy arrays) driving the GPU rhs and diag, against the oracle;
* Model.add_forcing (model.py:121-123, equations.py:229-238) with the
  forcing functions of tests/golden/forcings.py, static (a device field added
  in every stage) and time-dependent (formed on the host before each
  f2d_stage), against the reference's forced trajectories;
* innerproduct="classic" (operators.py:86-90) against the reference's
  fixtures (rsw, x-periodic euler, boussinesq).

Tolerance: 1e-10 relative L2 per field and per step, as the other FP64
parity tests.
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import fluids2d_gb300 as f2d  # noqa: E402
from fluids2d_gb300 import workloads as wl  # noqa: E402
from fluids2d_gb300._lib import lib  # noqa: E402
from test_gpu_parity import (MODEL_FILES, STEP_TOL, _model, _oracle_like,  # noqa: E402
                             compare, load, model_from_golden, rel_l2)

if GOLDEN not in sys.path:
    sys.path.insert(0, GOLDEN)
from forcings import BUILDERS as FORCINGS  # noqa: E402

FORCED = ["model_boussinesq_forced.npz", "model_qg_forced.npz",
          "model_euler_forced_time.npz", "model_rsw_forced_periodic.npz",
          "model_euler_forced_lfra.npz"]
# forcing functions that depend on neither time nor state
STATIC = {"buoyancy_rows", "wind_curl", "periodic_mass_source"}


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _forced_model(fname, static=None):
    g = load(fname)
    m = model_from_golden(g)
    name = str(g["forcing"])
    m.mesh.time = m.time
    st = (name in STATIC) if static is None else static
    m.add_forcing(FORCINGS[name](m), static=st)
    return g, m


def _rhs_vs_fixture(m, g):
    ds = m.new_prognostic()
    m.integrator.rhs(m.state, ds)
    worst = {}
    for name in ds._fields:
        v = getattr(ds, name)
        pairs = ((name + ".x", v.x), (name + ".y", v.y)) if hasattr(v, "x") else \
            ((name, v),)
        for key, got in pairs:
            ref = g["rhs0/" + key]
            fin = np.isfinite(ref)
            if not fin.all():
                # qgrsw: nan where the reference divides by a zero count of
                # wet vertices (land cells); the GPU writes 0 there
                assert not np.any(~fin & (m.mesh.msk > 0)), key
                got, ref = np.where(fin, got, 0.0), np.where(fin, ref, 0.0)
            if m.param.model == "qgrsw" and m.param.xperiodic:
                got, ref = got[:, 3:-3], ref[:, 3:-3]
            if not np.any(ref):
                assert not np.any(got), key
                continue
            worst[key] = rel_l2(got, ref)
    bad = {k: e for k, e in worst.items() if e > STEP_TOL}
    assert not bad, bad
    return worst


@pytest.mark.parametrize("fname", MODEL_FILES + FORCED)
def test_rhs_vs_reference(fname):
    g = load(fname)
    if "forcing" in g.files:
        g, m = _forced_model(fname)
    else:
        m = model_from_golden(g)
    _rhs_vs_fixture(m, g)
    # the state is untouched by rhs (qgrsw: pv/psi are its projection's work
    # arrays, as in the reference)
    m.sync()


def _steps_vs_fixture(m, g):
    getter = lambda pre: (lambda k: g[f"{pre}/{k}"] if f"{pre}/{k}" in g.files else None)  # noqa
    compare(m, getter("step0"), STEP_TOL)
    dts = g["dt"]
    for k in range(1, len(dts) + 1):
        m.advance(1)
        assert abs(m.time.dt - dts[k - 1]) <= 1e-10 * dts[k - 1]
        compare(m, getter(f"step{k}"), STEP_TOL)
    m.sync()
    assert abs(m.time.t - float(g["t"])) <= 1e-10 * float(g["t"])


@pytest.mark.parametrize("fname", FORCED)
def test_forced_steps_vs_reference(fname):
    g, m = _forced_model(fname)
    _steps_vs_fixture(m, g)


@pytest.mark.parametrize("fname", ["model_qg_forced.npz", "model_rsw_forced_periodic.npz"])
def test_static_forcing_through_stage_hook(fname):
    """A static forcing given as a per-stage function (f2d_stage path) gives
    the same trajectory as the device field path."""
    g, m = _forced_model(fname, static=False)
    _steps_vs_fixture(m, g)


def test_forcing_set_refuses_unknown_variable():
    m = _model("eulerpsi", 32, 32)
    a = np.zeros(m.mesh.shape)
    rc = lib().f2d_forcing_set(m._h, b"u.x", a.ctypes.data)
    assert rc != 0 and b"no prognostic variable" in lib().f2d_last_error()


def test_stage_out_of_range():
    m = _model("eulerpsi", 32, 32, integrator="ef")
    assert lib().f2d_stage(m._h, 2) != 0
    assert b"out of range" in lib().f2d_last_error()


def _addto(y, terms):
    """addto_list (integrators.py:175-196) on host arrays: y += sum c x."""
    for name in y._fields:
        v = getattr(y, name)
        if hasattr(v, "x"):
            for comp in ("x", "y"):
                acc = getattr(v, comp)
                inc = sum(c * getattr(getattr(x, name), comp) for c, x in terms)
                acc += inc
        else:
            v += sum(c * getattr(x, name) for c, x in terms)


class _ProgView:
    """The prognostic part of the model's host state, for _addto."""

    def __init__(self, m):
        from fluids2d_gb300.model import _specs
        _, prog = _specs(m.param)
        self._fields = prog
        st = m.state
        for n in prog:
            setattr(self, n, getattr(st, n))


@pytest.mark.parametrize("kind", ["eulerpsi", "rsw", "qgrsw"])
def test_reference_rk3_loop_drives_gpu_rhs(kind):
    """The reference's rk3 (integrators.py:92-107) as a host loop over the
    GPU plug points: rhs(s, ds) and diag(s) from get_rhs_and_diag, addto on
    the host arrays. Three steps against the oracle."""
    if kind == "eulerpsi":
        case = wl.eulerpsi_case(n=64, ny=48, seed=3, nislands=2)
        extra = dict(cfl=0.8)
    elif kind == "rsw":
        case = wl.rsw_case(n=64, ny=48, seed=4, nislands=2)
        extra = {}
    else:
        case = wl.rsw_case(n=48, ny=40, seed=9, nislands=2, xperiodic=False, f0=10.0)
        z = np.zeros_like(case["fields"]["h"])
        case["fields"] = {"u.x": z, "u.y": z.copy(), "h": case["fields"]["h"]}
        extra = dict(cfl=0.5)
    om = _oracle_like(case, kind, **extra)
    kw = dict(xperiodic=case.get("xperiodic", False), Lx=case["Lx"], Ly=case["Ly"],
              tend=1e300, maxite=10 ** 9, **extra)
    for k in ("f0", "g", "H", "beta"):
        if k in case:
            kw[k] = case[k]
    m = _model(kind, case["nx"], case["ny"], case["msk"], **kw)
    s = m.state
    for k, v in case["fields"].items():
        if "." in k:
            getattr(getattr(s, k.split(".")[0]), k.split(".")[1])[:] = v
        else:
            getattr(s, k)[:] = v
    if kind == "qgrsw":
        from oracle import oracle as O
        O.qg_projection(om.mesh, om.s["u.x"], om.s["u.y"], om.s["h"], om.s["pv"],
                        om.s["psi"])
        om.diag()
        m.qg_projection()
    integ = m.integrator
    integ.diag(m.state)
    ds1, ds2, ds3 = (m.new_prognostic() for _ in range(3))
    for _ in range(3):
        om.run_steps(1)
        m.set_dt()
        dt = m.time.dt
        assert abs(dt - om.dt) <= 1e-10 * om.dt
        integ.rhs(m.state, ds1)
        _addto(_ProgView(m), [(dt, ds1)])
        integ.diag(m.state)
        integ.rhs(m.state, ds2)
        _addto(_ProgView(m), [(-3 * dt / 4, ds1), (dt / 4, ds2)])
        integ.diag(m.state)
        integ.rhs(m.state, ds3)
        _addto(_ProgView(m), [(-dt / 12, ds1), (-dt / 12, ds2), (2 * dt / 3, ds3)])
        integ.diag(m.state)
        compare(m, lambda k: om.s.get(k), STEP_TOL)
    m.sync()


@pytest.mark.parametrize("fname", ["model_rsw_classic.npz",
                                   "model_euler_classic_periodic.npz",
                                   "model_boussinesq_classic.npz"])
def test_classic_innerproduct_vs_reference(fname):
    g = load(fname)
    m = model_from_golden(g)
    assert m.param.innerproduct == "classic"
    _steps_vs_fixture(m, g)
    assert os.path.basename(fname) in MODEL_FILES
