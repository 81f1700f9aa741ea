"""Pin the oracle against outputs of the reference itself.

The fixtures in tests/golden/ were produced by the unmodified reference
(``make_golden.py``). Integer/mask outputs must match exactly; the flux
sweeps, which the oracle restates expression by expression, must match bit for
bit; solver and whole-step outputs are compared to 1e-13 relative (SuperLU is
the same library on both sides, the tolerance only covers a different scipy
build on another machine).
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as O

if GOLDEN not in sys.path:
    sys.path.insert(0, GOLDEN)
from forcings import BUILDERS as FORCINGS  # noqa: E402


def load(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def _noslip(s):
    """param.noslip from the text the generator wrote: None, True, False or
    a list of side names such as "['left', 'top']"."""
    text = str(s)
    fixed = {"None": None, "True": True, "False": False}
    if text in fixed:
        return fixed[text]
    if text.startswith("[") and text.endswith("]"):
        return [w.strip().strip("'\"") for w in text[1:-1].split(",") if w.strip()]
    raise ValueError(f"unexpected noslip fixture value {text!r}")


@pytest.mark.parametrize("case", list(load("mesh.npz")["names"]))
def test_mesh_bitexact(case):
    g = load("mesh.npz")
    nx, ny, xper, maxo = (int(v) for v in g[case + "/params"])
    p = O.Param(model="eulerpsi", nx=nx, ny=ny, xperiodic=bool(xper),
                maxorder=maxo, noslip=_noslip(g[case + "/noslip"]))
    m = O.Mesh.__new__(O.Mesh)
    # build like Mesh.__init__ but with the golden mask, without solvers
    m.param = p
    m.shape = (ny + 6, nx + 6)
    m.xshift, m.yshift = 1, nx + 6
    m.msk = g[case + "/msk"].copy()
    m.set_masks()
    for k in ("mskx", "msky", "mskv"):
        np.testing.assert_array_equal(getattr(m, k), g[case + "/" + k], k)
    sc = O.slipcoef(p, m.msk)
    np.testing.assert_array_equal(sc, g[case + "/slipcoef"])
    mv = (1 * (sc > 0)).astype(np.int8)
    orders = {
        "ocx": O.set_order(m.msk, 1, maxo),
        "ocy": O.set_order(m.msk, nx + 6, maxo),
        "ovx": O.set_order(mv, -1, maxo) * m.msky,
        "ovy": O.set_order(mv, -(nx + 6), maxo) * m.mskx,
        "okx": O.set_order(m.mskx, -1, maxo),
        "oky": O.set_order(m.msky, -(nx + 6), maxo),
    }
    for k, v in orders.items():
        np.testing.assert_array_equal(v, g[case + "/" + k], k)
    np.testing.assert_array_equal(O.gindex(O.vertex_msk(m, "c")),
                                  g[case + "/Gc"])
    np.testing.assert_array_equal(O.gindex(O.vertex_msk(m, "v")),
                                  g[case + "/Gv"])


@pytest.mark.parametrize("method", ["weno", "upwind", "centered", "cweno"])
def test_sweeps_bitexact(method):
    g = load("sweeps.npz")
    q, U, V = g["q"], g["U"], g["V"]
    sx, sy = (int(v) for v in g["shifts"])
    for d, s, s2, sign in (("x", sx, sy, -1), ("y", sy, sx, +1)):
        flx = np.zeros_like(q)
        O.compflux(flx, U, q, g["oc" + d], s, method, pysq=True)
        np.testing.assert_array_equal(flx, g[f"compflux/{method}/{d}"])
        du = np.zeros_like(q)
        O.vortexforce(du, V, q, g["ov" + d], s, s2, sign, method, pysq=True)
        np.testing.assert_array_equal(du, g[f"vortexforce/{method}/{d}"])
        ke = g[f"innerproduct_in/{method}/{d}"].copy()
        O.innerproduct(ke, U, q, g["ok" + d], s, method, pysq=True)
        np.testing.assert_array_equal(ke, g[f"innerproduct/{method}/{d}"])


def test_sweeps_numba_square_close():
    """The x*x entry points (numba semantics) differ by rounding only."""
    g = load("sweeps.npz")
    q, U = g["q"], g["U"]
    flx = np.zeros_like(q)
    O.compflux(flx, U, q, g["ocx"], 1, "weno", pysq=False)
    ref = g["compflux/weno/x"]
    assert np.max(np.abs(flx - ref)) <= 1e-13 * np.max(np.abs(ref))


@pytest.mark.parametrize("case", list(load("poisson.npz")["names"]))
def test_poisson_vs_reference(case):
    g = load("poisson.npz")
    nx, ny, xper = (int(v) for v in g[case + "/params"])
    f0 = float(g[case + "/f0"])
    model = "qg" if float(g[case + "/maindiag"]) != 0 else "eulerpsi"
    p = O.Param(model=model, nx=nx, ny=ny, xperiodic=bool(xper), f0=f0)
    m = O.Model(p, msk=g[case + "/msk"])
    solver = m.mesh.qg_helmholtz if model == "qg" else m.mesh.poisson_vertices
    if model == "qg":
        assert m.mesh.maindiag == float(g[case + "/maindiag"])
    x = g[case + "/x0"].copy()
    solver.solve(g[case + "/b"], x)
    ref = g[case + "/x"]
    assert np.max(np.abs(x - ref)) <= 1e-13 * np.max(np.abs(ref))


MODEL_FILES = ["model_eulerpsi.npz", "model_eulerpsi_islands.npz",
               "model_rsw.npz", "model_qg.npz", "model_eulerpsi_ef.npz",
               "model_eulerpsi_enrk3.npz", "model_rsw_enrk3.npz",
               "model_euler.npz", "model_euler_periodic.npz",
               "model_eulerpsi_lfra.npz", "model_qg_lfra.npz", "model_rsw_lfra.npz",
               "model_euler_lfra_periodic.npz", "model_boussinesq.npz",
               "model_boussinesq_periodic.npz", "model_boussinesq_lfra.npz",
               "model_eulerpsi_tracer.npz", "model_qg_tracer_lfra.npz",
               "model_rsw_tracer.npz", "model_boussinesq_tracer.npz",
               "model_qgrsw.npz", "model_qgrsw_periodic.npz", "model_qgrsw_lfra.npz",
               "model_qgrsw_tracer.npz", "model_rsw_classic.npz",
               "model_euler_classic_periodic.npz", "model_boussinesq_classic.npz",
               "model_boussinesq_forced.npz", "model_qg_forced.npz",
               "model_euler_forced_time.npz", "model_rsw_forced_periodic.npz",
               "model_euler_forced_lfra.npz"]


def oracle_from_golden(g, pysq=True):
    nx, ny, xper = (int(v) for v in g["params"])
    Lx, Ly, f0, beta, gg, H, cfl = (float(v) for v in g["scalars"])
    model = [k for k in g.files if k.startswith("ic/")]
    names = {k[3:] for k in model}
    kind = (str(g["model"]) if "model" in g.files else
            "eulerpsi" if "omega" in names else
            "rsw" if "h" in names else "boussinesq" if "b" in names else
            "euler" if "u.x" in names else "qg")
    integ = str(g["integrator"]) if "integrator" in g.files else "rk3"
    gam = float(g["RAgamma"]) if "RAgamma" in g.files else 0.1
    tracer = str(g["tracer"]) if "tracer" in g.files else None
    ip = str(g["innerproduct"]) if "innerproduct" in g.files else "weno"
    p = O.Param(model=kind, nx=nx, ny=ny, xperiodic=bool(xper), Lx=Lx, Ly=Ly,
                f0=f0, beta=beta, g=gg, H=H, cfl=cfl, tend=1e9,
                maxite=10 ** 9, integrator=integ, RAgamma=gam, tracer=tracer,
                innerproduct=ip)
    m = O.Model(p, msk=g["msk"], pysq=pysq)
    if "f" in g.files:
        m.mesh.f = g["f"].copy()
    if "forcing" in g.files:
        m.mesh.time = m  # forcing functions read mesh.time.t
        m.add_forcing(FORCINGS[str(g["forcing"])](m))
    for k in names:
        m.s[k][:] = g["ic/" + k]
    m.diag()
    return m


def _compare_state(m, g, prefix, tol):
    worst = 0.0
    for k, v in m.s.items():
        ref = g[f"{prefix}/{k}"]
        # the reference writes nan where qg_projection divides by a zero
        # count of wet vertices (land cells): same places, finite elsewhere
        fin = np.isfinite(ref)
        np.testing.assert_array_equal(np.isfinite(v), fin, err_msg=f"{prefix} {k}")
        v, ref = v[fin], ref[fin]
        scale = max(np.max(np.abs(ref)), 1e-300)
        err = np.max(np.abs(v - ref)) / scale
        assert err <= tol, (prefix, k, err)
        worst = max(worst, err)
    return worst


@pytest.mark.parametrize("fname", MODEL_FILES)
def test_model_steps_vs_reference(fname):
    g = load(fname)
    m = oracle_from_golden(g)
    _compare_state(m, g, "step0", 1e-13)
    # one rhs evaluation on the initial state
    ds = {k: np.zeros_like(v) for k, v in m.scratch[0].items()}
    m.rhs(m.s, ds)
    for k, v in ds.items():
        ref = g["rhs0/" + k]
        fin = np.isfinite(ref)
        np.testing.assert_array_equal(np.isfinite(v), fin, err_msg=k)
        v, ref = v[fin], ref[fin]
        assert np.max(np.abs(v - ref)) <= 1e-13 * max(np.max(np.abs(ref)),
                                                       1e-300), k
    dts = g["dt"]
    for k in range(1, len(dts) + 1):
        m.set_dt()
        assert abs(m.dt - dts[k - 1]) <= 1e-13 * dts[k - 1]
        m.step(1)
        _compare_state(m, g, f"step{k}", 1e-12)
    assert abs(m.t - float(g["t"])) <= 1e-13 * float(g["t"])


@pytest.mark.parametrize("fname", ["bulk_rsw.npz", "bulk_euler.npz"])
def test_bulk_diagnostics_vs_reference(fname):
    """diagnostics.py:39-57 along 7 steps (records at ite 0, 3, 6)."""
    g = load(fname)
    m = oracle_from_golden(g)
    recs = [O.bulk(m)]
    for k, dt in enumerate(g["dt"], start=1):
        m.set_dt()
        assert abs(m.dt - dt) <= 1e-13 * dt
        m.step(1)
        if m.ite % 3 == 0:
            recs.append(O.bulk(m))
    ref = g["bulk"]
    got = np.array(recs)
    assert got.shape == ref.shape
    for c in range(5):
        scale = max(np.abs(ref[:, c]).max(), 1e-300)
        assert np.abs(got[:, c] - ref[:, c]).max() <= 1e-12 * scale, c


@pytest.mark.parametrize("fname", ["model_qgrsw.npz", "model_qgrsw_periodic.npz",
                                   "model_qgrsw_tracer.npz"])
def test_qg_projection_state_form_vs_reference(fname):
    """qg_projection (operators.py:176-183, anomaly=False) of the state the
    reference applied it to (pre/...) against the state it left (ic/...),
    nan where the reference divides by a zero count of wet vertices."""
    g = load(fname)
    m = oracle_from_golden(g)
    s = m.s
    for k in ("u.x", "u.y", "h", "pv", "psi"):
        s[k][:] = g["pre/" + k]
    O.qg_projection(m.mesh, s["u.x"], s["u.y"], s["h"], s["pv"], s["psi"])
    for k in ("u.x", "u.y", "h", "pv", "psi"):
        ref = g["ic/" + k]
        fin = np.isfinite(ref)
        np.testing.assert_array_equal(np.isfinite(s[k]), fin, err_msg=k)
        scale = max(np.abs(ref[fin]).max(), 1e-300)
        assert np.abs(s[k][fin] - ref[fin]).max() <= 1e-12 * scale, k
