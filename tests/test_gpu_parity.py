"""GPU parity: the CUDA path against the reference (golden fixtures) and the
oracle, through the C ABI.

Tolerances (FP64 form): flux sweeps 1e-13 relative to the array's max (the
kernels may contract multiply-adds into FMAs, the reference does not);
Poisson/Helmholtz solves 1e-10 relative L2 (multigrid-PCG to a relative
residual of 1e-12 against the reference's direct LU); whole model states
1e-10 relative L2 per field and per step.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import fluids2d_gb300 as f2d  # noqa: E402
from fluids2d_gb300 import _lib, workloads as wl  # noqa: E402

SWEEP_TOL = 1e-13
SOLVE_TOL = 1e-10
STEP_TOL = 1e-10


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def load(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    d = np.linalg.norm(a - b)
    return d / nb if nb > 0 else d


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def dptr(t):
    return _lib.c_void_p(t.data_ptr())


# ------------------------------------------------------------- sweeps ----
@pytest.mark.parametrize("method", ["weno", "upwind", "centered", "cweno"])
def test_sweeps_vs_reference(method):
    g = load("sweeps.npz")
    L = _lib.lib()
    M = _lib.METHODS[method]
    q, U, V = dev(g["q"]), dev(g["U"]), dev(g["V"])
    sx, sy = (int(v) for v in g["shifts"])
    n = g["q"].size
    for d, s, s2, sign in (("x", sx, sy, -1), ("y", sy, sx, +1)):
        o = dev(g["oc" + d])
        flx = torch.zeros_like(q)
        _lib.check(L.f2d_compflux(M, dptr(flx), dptr(U), dptr(q), dptr(o), s, 0,
                                  n, None))
        ref = g[f"compflux/{method}/{d}"]
        torch.cuda.synchronize()
        assert np.max(np.abs(flx.cpu().numpy() - ref)) <= SWEEP_TOL * np.max(np.abs(ref))
        o = dev(g["ov" + d])
        du = torch.zeros_like(q)
        _lib.check(L.f2d_vortexforce(M, dptr(du), dptr(V), dptr(q), dptr(o), s, s2,
                                     sign, 0, n, None))
        ref = g[f"vortexforce/{method}/{d}"]
        torch.cuda.synchronize()
        assert np.max(np.abs(du.cpu().numpy() - ref)) <= SWEEP_TOL * np.max(np.abs(ref))
        o = dev(g["ok" + d])
        ke = dev(g[f"innerproduct_in/{method}/{d}"])
        _lib.check(L.f2d_innerproduct(M, dptr(ke), dptr(U), dptr(q), dptr(o), s, 0,
                                      n, None))
        ref = g[f"innerproduct/{method}/{d}"]
        torch.cuda.synchronize()
        assert np.max(np.abs(ke.cpu().numpy() - ref)) <= SWEEP_TOL * np.max(np.abs(ref))


# ------------------------------------------------------------ poisson ----
def _model(kind, nx, ny, msk=None, **kw):
    p = f2d.Param()
    p.model = kind
    p.nx, p.ny = nx, ny
    for k, v in kw.items():
        setattr(p, k, v)
    m = f2d.Model(p)
    if msk is not None:
        m.mesh.msk[:] = msk
        m.mesh.finalize()
    return m


@pytest.mark.parametrize("case", list(load("poisson.npz")["names"]))
def test_poisson_vs_reference(case):
    g = load("poisson.npz")
    nx, ny, xper = (int(v) for v in g[case + "/params"])
    helm = float(g[case + "/maindiag"]) != 0
    m = _model("qg" if helm else "eulerpsi", nx, ny, g[case + "/msk"],
               xperiodic=bool(xper), f0=float(g[case + "/f0"]))
    solver = m.mesh.qg_helmholtz if helm else m.mesh.poisson_vertices
    x = g[case + "/x0"].copy()
    solver.solve(g[case + "/b"], x)
    ref = g[case + "/x"]
    assert rel_l2(x, ref) <= SOLVE_TOL, (rel_l2(x, ref), solver.last_iters)
    # points the reference does not write keep their values
    touched = (m.mesh.G_vertices >= 0)
    if xper:
        touched[:, :3] = touched[:, -3:] = True
    np.testing.assert_array_equal(x[~touched], g[case + "/x0"][~touched])


def test_poisson_zero_rhs():
    m = _model("eulerpsi", 24, 20)
    x = np.random.default_rng(0).normal(size=m.mesh.shape)
    m.mesh.poisson_vertices.solve(np.zeros(m.mesh.shape), x)
    assert np.all(x[m.mesh.G_vertices >= 0] == 0)


# -------------------------------------------------------------- models ----
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
               "model_euler_classic_periodic.npz", "model_boussinesq_classic.npz"]


def model_from_golden(g):
    nx, ny, xper = (int(v) for v in g["params"])
    Lx, Ly, f0, beta, gg, H, cfl = (float(v) for v in g["scalars"])
    names = {k[3:] for k in g.files if k.startswith("ic/")}
    kind = (str(g["model"]) if "model" in g.files else
            "eulerpsi" if "omega" in names else "rsw" if "h" in names else
            "boussinesq" if "b" in names else
            "euler" if "u.x" in names else "qg")
    integ = str(g["integrator"]) if "integrator" in g.files else "rk3"
    gam = float(g["RAgamma"]) if "RAgamma" in g.files else 0.1
    tracer = str(g["tracer"]) if "tracer" in g.files else None
    ip = str(g["innerproduct"]) if "innerproduct" in g.files else "weno"
    m = _model(kind, nx, ny, g["msk"], xperiodic=bool(xper), Lx=Lx, Ly=Ly, f0=f0,
               beta=beta, g=gg, H=H, cfl=cfl, tend=1e300, maxite=10 ** 9,
               integrator=integ, RAgamma=gam, tracer=tracer, innerproduct=ip)
    if "f" in g.files:
        m.mesh.f = g["f"]
    s = m.state
    for k in names:
        if "." in k:
            getattr(getattr(s, k.split(".")[0]), k.split(".")[1])[:] = g["ic/" + k]
        else:
            getattr(s, k)[:] = g["ic/" + k]
    m.integrator.diag(s)
    return m


def state_dict(m):
    out = {}
    s = m.state
    for name in s._fields:
        v = getattr(s, name)
        if hasattr(v, "_fields"):
            out[name + ".x"], out[name + ".y"] = v.x.copy(), v.y.copy()
        else:
            out[name] = v.copy()
    return out


def compare(m, ref_get, tol, skip=("flx.x", "flx.y")):
    worst = {}
    for k, v in state_dict(m).items():
        if k in skip:
            continue
        r = ref_get(k)
        if r is None:
            continue
        fin = np.isfinite(r)
        if not fin.all():
            # qgrsw: the reference's thickness_from_psi writes nan ((1/0)*0)
            # into cells without a wet vertex (land); the GPU writes 0 there
            fl = (m.mesh.mskv if k in ("pv", "psi") else m.mesh.msk) > 0
            assert not np.any(~fin & fl), k
            v, r = np.where(fin, v, 0.0), np.where(fin, r, 0.0)
        if m.param.model == "qgrsw" and m.param.xperiodic and k == "pv":
            # x-periodic qgrsw: the PV of the halo columns is formed from the
            # raw tendency before its fill, whose last column the reference's
            # div (operators.py:104-107) leaves at the scratch array's
            # previous content; the PV of the interior vertices (the solve's
            # right-hand side) is compared
            v, r = v[:, 3:-3], r[:, 3:-3]
        if not np.any(r):
            continue
        if m.param.model in ("euler", "boussinesq") and k == "p":
            # the Neumann pressure is defined up to a constant: compare the
            # zero-mean parts over the fluid cells
            fl = m.mesh.msk > 0
            if m.param.xperiodic:
                fl[:, :3] = False
                fl[:, -3:] = False
            v = np.where(fl, v - v[fl].mean(), 0.0)
            r = np.where(fl, r - r[fl].mean(), 0.0)
        worst[k] = rel_l2(v, r)
    bad = {k: e for k, e in worst.items() if e > tol}
    assert not bad, bad
    return worst


@pytest.mark.parametrize("fname", MODEL_FILES)
def test_model_steps_vs_reference(fname):
    g = load(fname)
    m = model_from_golden(g)
    getter = lambda pre: (lambda k: g[f"{pre}/{k}"] if f"{pre}/{k}" in g.files else None)  # noqa
    compare(m, getter("step0"), STEP_TOL)
    dts = g["dt"]
    for k in range(1, len(dts) + 1):
        m.advance(1)
        assert abs(m.time.dt - dts[k - 1]) <= 1e-10 * dts[k - 1]
        compare(m, getter(f"step{k}"), STEP_TOL)
    m.sync()
    assert abs(m.time.t - float(g["t"])) <= 1e-10 * float(g["t"])
    assert m.time.ite == len(dts)


def _oracle_like(case, kind, **extra):
    p = O.Param(model=kind, nx=case["nx"], ny=case["ny"],
                xperiodic=case.get("xperiodic", False), Lx=case["Lx"],
                Ly=case["Ly"], tend=1e300, maxite=10 ** 9, **extra)
    for k in ("f0", "g", "H", "beta"):
        if k in case:
            setattr(p, k, case[k])
    om = O.Model(p, msk=case["msk"], pysq=False)
    if "f" in case:
        om.mesh.f = case["f"].copy()
    for k, v in case["fields"].items():
        om.s[k][:] = v
    om.diag()
    return om


@pytest.mark.parametrize("kind", ["eulerpsi", "rsw", "qg", "euler", "boussinesq"])
def test_model_vs_oracle_larger(kind):
    if kind == "euler":
        case = wl.euler_case(n=128, ny=96, seed=5, nislands=3)
    elif kind == "boussinesq":
        case = wl.boussinesq_case(n=128, ny=96, seed=5, nislands=3)
    elif kind == "eulerpsi":
        case = wl.eulerpsi_case(n=128, ny=96, seed=5, nislands=3)
    elif kind == "rsw":
        case = wl.rsw_case(n=128, ny=96, seed=6, nislands=3)
    else:
        case = wl.qg_case(n=128, ny=128, seed=7, nislands=4)
    om = _oracle_like(case, kind)
    kw = dict(xperiodic=case.get("xperiodic", False), Lx=case["Lx"], Ly=case["Ly"],
              tend=1e300, maxite=10 ** 9)
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
    compare(m, lambda k: om.s.get(k), STEP_TOL)
    for _ in range(4):
        om.run_steps(1)
        m.advance(1)
        assert abs(m.time.dt - om.dt) <= 1e-10 * om.dt
        compare(m, lambda k: om.s.get(k), STEP_TOL)
    m.sync()


@pytest.mark.parametrize("kind", ["eulerpsi", "rsw", "boussinesq"])
@pytest.mark.parametrize("method", ["upwind", "centered", "cweno"])
def test_model_flux_methods_vs_oracle(kind, method):
    """The fused stage kernels with the reference's other flux methods
    (weno.py:338-343): whole steps against the oracle."""
    if kind == "eulerpsi":
        case = wl.eulerpsi_case(n=64, ny=48, seed=15, nislands=2)
        extra = dict(compflux=method)
    elif kind == "boussinesq":
        case = wl.boussinesq_case(n=64, ny=48, seed=17, nislands=2)
        extra = dict(compflux=method, vortexforce=method, innerproduct=method)
    else:
        case = wl.rsw_case(n=64, ny=48, seed=16, nislands=2)
        extra = dict(compflux=method, vortexforce=method, innerproduct=method)
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
    m.integrator.diag(s)
    for _ in range(3):
        om.run_steps(1)
        m.advance(1)
        assert abs(m.time.dt - om.dt) <= 1e-10 * om.dt
        compare(m, lambda k: om.s.get(k), STEP_TOL)
    m.sync()


@pytest.mark.parametrize("xper", [False, True])
def test_qgrsw_projection_and_steps_vs_oracle(xper):
    """qgrsw at 128x96 with islands: the state-form qg_projection (the
    reference's initialisation, operators.py:176-183) on the GPU against the
    oracle's, then whole steps."""
    from fluids2d_gb300.operators import qg_projection
    case = wl.rsw_case(n=128, ny=96, seed=9, nislands=3, xperiodic=xper, f0=10.0)
    z = np.zeros_like(case["fields"]["h"])
    case["fields"] = {"u.x": z, "u.y": z.copy(), "h": case["fields"]["h"]}
    om = _oracle_like(case, "qgrsw", cfl=0.5)
    O.qg_projection(om.mesh, om.s["u.x"], om.s["u.y"], om.s["h"], om.s["pv"],
                    om.s["psi"])
    om.diag()
    m = _model("qgrsw", case["nx"], case["ny"], case["msk"], xperiodic=xper,
               Lx=case["Lx"], Ly=case["Ly"], f0=case["f0"], g=case["g"], H=case["H"],
               cfl=0.5, tend=1e300, maxite=10 ** 9)
    s = m.state
    s.u.x[:] = case["fields"]["u.x"]
    s.u.y[:] = case["fields"]["u.y"]
    s.h[:] = case["fields"]["h"]
    qg_projection(m.mesh, s.u, s.h, s.pv, s.psi)
    m.integrator.diag(m.state)
    compare(m, lambda k: om.s.get(k), STEP_TOL)
    for _ in range(4):
        om.run_steps(1)
        m.advance(1)
        assert abs(m.time.dt - om.dt) <= 1e-10 * om.dt
        compare(m, lambda k: om.s.get(k), STEP_TOL)
    m.sync()


@pytest.mark.parametrize("fname", ["bulk_rsw.npz", "bulk_euler.npz"])
def test_bulk_diagnostics_vs_reference(fname, tmp_path):
    """Bulk (diagnostics.py:39-57) reduced on the GPU into the device ring
    along the reference's trajectory: records at ite 0, 3, 6."""
    from fluids2d_gb300.diagnostics import Bulk
    g = load(fname)
    m = model_from_golden(g)
    b = Bulk(m, ncfile=str(tmp_path / "bulk.nc"))
    m.diags.append(b)
    b()
    for _ in range(len(g["dt"])):
        m.advance(1)
        m.compute_diags()
    b.finalize()
    data = b.read()
    got = np.stack([getattr(data, n) for n in Bulk.variables], axis=1)
    ref = g["bulk"]
    assert got.shape == ref.shape
    for c in range(5):
        scale = max(np.abs(ref[:, c]).max(), 1e-300)
        assert np.abs(got[:, c] - ref[:, c]).max() <= 1e-10 * scale, (c, got[:, c], ref[:, c])


def test_history_float32_snapshots(tmp_path):
    """Model.run with nhis: t, ite, dt and var_to_store as float32 records
    (io.py:12-21, dtype "f"), every nhis iterations and at the end."""
    case = wl.rsw_case(n=64, ny=48, seed=2, nislands=2)
    m = _model("rsw", 64, 48, case["msk"], xperiodic=True, tend=1e300, maxite=7,
               nhis=3, var_to_store=["h", "u"], outputfile=str(tmp_path / "hist.nc"))
    m.state.h[:] = case["fields"]["h"]
    m.integrator.diag(m.state)
    m.run()
    f = np.load(tmp_path / "hist.npz")
    assert list(f["ite"]) == [0, 3, 6, 7]
    assert f["h"].dtype == np.float32 and f["h"].shape == (4, 54, 70)
    np.testing.assert_array_equal(f["h"][-1], m.state.h.astype(np.float32))
    np.testing.assert_array_equal(f["ux"][-1], m.state.u.x.astype(np.float32))
    assert abs(float(f["t"][-1]) - np.float32(m.time.t)) == 0


# --------------------------------------------- size-independent checks ----
def test_tracer_constant_and_conserved_periodic():
    """x-periodic boussinesq channel at 256^2 with a passive tracer: a tracer
    that is 1 on every fluid cell stays 1 under the divergence-free flow (to
    the projection's tolerance), and its total over the fluid cells is
    conserved to round-off."""
    case = wl.boussinesq_case(n=256, seed=24, nislands=3, xperiodic=True)
    m = _model("boussinesq", 256, 256, case["msk"], xperiodic=True, cfl=0.5,
               tend=1e300, maxite=10 ** 9, tracer="q")
    s = m.state
    for k, v in case["fields"].items():
        if "." in k:
            getattr(getattr(s, k.split(".")[0]), k.split(".")[1])[:] = v
        else:
            getattr(s, k)[:] = v
    s.q[:] = case["msk"].astype(np.float64)
    m.integrator.diag(s)
    fl = m.mesh.msk > 0
    fl[:, :3] = False
    fl[:, -3:] = False
    q0 = float(np.sum(m.state.q[fl]))
    m.advance(8)
    m.sync()
    q = m.state.q
    assert np.abs(q[fl] - 1.0).max() <= 1e-8
    assert abs(float(np.sum(q[fl])) - q0) <= 1e-12 * q0
    # the flow moved (the buoyancy field changed)
    assert rel_l2(m.state.b, case["fields"]["b"]) > 1e-4


def test_boussinesq_buoyancy_conservation_full_size():
    """Closed basin with islands at 512^2: the flux-form buoyancy equation
    conserves the total buoyancy (sum over the fluid cells) to round-off,
    and the projected velocity stays divergence-free."""
    case = wl.boussinesq_case(n=512, seed=23, nislands=4)
    m = _model("boussinesq", 512, 512, case["msk"], cfl=0.5, tend=1e300,
               maxite=10 ** 9)
    s = m.state
    for k, v in case["fields"].items():
        if "." in k:
            getattr(getattr(s, k.split(".")[0]), k.split(".")[1])[:] = v
        else:
            getattr(s, k)[:] = v
    m.integrator.diag(s)
    fl = m.mesh.msk > 0
    b0 = float(np.sum(m.state.b[fl]))
    babs = float(np.sum(np.abs(m.state.b[fl])))
    m.advance(10)
    m.sync()
    s = m.state
    assert abs(float(np.sum(s.b[fl])) - b0) <= 1e-12 * babs
    Ux, Uy = s.U.x, s.U.y
    d = np.zeros_like(Ux)
    d[:, :-1] = -np.diff(Ux, axis=1)
    d[:-1, :] -= np.diff(Uy, axis=0)
    scale = np.abs(Ux).max() + np.abs(Uy).max()
    assert np.abs(d[fl]).max() <= 1e-9 * scale
    # buoyancy did work: the state moved
    assert rel_l2(s.b, case["fields"]["b"]) > 1e-4


@pytest.mark.parametrize("xper", [False, True])
def test_euler_projection_divergence_free(xper):
    """After the pressure projection the discrete divergence of U vanishes at
    every fluid cell (to the solve's tolerance), at 256^2 with islands."""
    case = wl.euler_case(n=256, seed=21, nislands=4, xperiodic=xper)
    m = _model("euler", 256, 256, case["msk"], xperiodic=xper, cfl=0.5, tend=1e300,
               maxite=10 ** 9)
    s = m.state
    s.u.x[:] = case["fields"]["u.x"]
    s.u.y[:] = case["fields"]["u.y"]
    m.integrator.diag(s)
    m.advance(3)
    m.sync()
    s = m.state
    Ux, Uy = s.U.x, s.U.y
    d = np.zeros_like(Ux)
    d[:, :-1] = -np.diff(Ux, axis=1)
    d[:-1, :] -= np.diff(Uy, axis=0)
    fl = m.mesh.msk > 0
    if xper:
        fl[:, :3] = False
        fl[:, -3:] = False
    scale = np.abs(Ux).max() + np.abs(Uy).max()
    assert np.abs(d[fl]).max() <= 1e-9 * scale
    # the pre-projection divergence (state "div") was not small
    assert np.abs(s.div[fl]).max() > 1e-6 * scale


# --------------------------------------------- size-independent checks (cont.) ----
def test_rsw_mass_conservation_full_size():
    case = wl.rsw_case(n=512, seed=0, nislands=3)
    m = _model("rsw", 512, 512, case["msk"], xperiodic=True, f0=1.0, g=1, H=1,
               tend=1e300, maxite=10 ** 9)
    m.state.h[:] = case["fields"]["h"]
    m.integrator.diag(m.state)
    inner = (slice(3, -3), slice(3, -3))
    mass0 = float(np.sum(m.state.h[inner]))
    m.advance(20)
    m.sync()
    mass1 = float(np.sum(m.state.h[inner]))
    assert abs(mass1 - mass0) <= 1e-12 * abs(mass0)
    assert np.all(np.isfinite(m.state.u.x))


def test_eulerpsi_circulation_full_size():
    case = wl.eulerpsi_case(n=256, seed=0)
    m = _model("eulerpsi", 256, 256, case["msk"], cfl=0.8, tend=1e300,
               maxite=10 ** 9)
    m.state.omega[:] = case["fields"]["omega"]
    m.integrator.diag(m.state)
    w0 = m.state.omega.copy()
    m.advance(10)
    m.sync()
    w1 = m.state.omega
    assert abs(w1.sum() - w0.sum()) <= 1e-12 * np.abs(w0).sum()
    # the Poisson solve of the last diagnostic is converged
    psi = m.state.psi
    lap = O.laplacian(O.Mesh(O.Param(model="eulerpsi", nx=256, ny=256)), 0)[0]
    G = m.mesh.G_vertices
    sel = G >= 0
    b = m.state.vomega[sel]
    r = b - lap @ psi[sel]
    assert np.linalg.norm(r) <= 1e-10 * np.linalg.norm(b)


def test_poisson_maxit_reports_status():
    m = _model("eulerpsi", 64, 64, poisson_maxit=1, poisson_tol=1e-15)
    case = wl.eulerpsi_case(n=64, seed=1)
    m.state.omega[:] = case["fields"]["omega"]
    m.integrator.diag(m.state)
    with pytest.raises(f2d.F2DError, match="max iterations"):
        m.sync()
    m.sync()  # status is cleared once reported


# ------------------------------------------------ FP32 + FP64 refinement ----
# Stencils, RK3 state and the multigrid cycle in FP32; the Poisson solution
# refined to FP64 accuracy by the FP64 CG residual recurrence. The solve
# itself must match SuperLU to the FP64 tolerance; model states match the
# FP64 oracle within FP32 rounding accumulated over 5 steps: 1e-6 relative
# L2 for eulerpsi and qg (the target of the FP32 form); 1e-4 for rsw, euler
# and boussinesq, whose velocity is driven by the gradient of p = g h / area
# ~ 1 (rsw) or by a pressure from an FP32 divergence, with O(1e-3) anomalies,
# so the FP32 rounding of p (6e-8) is amplified ~1e3 by the cancellation in
# grad p.
FP32_STATE_TOL = {"eulerpsi": 1e-6, "qg": 1e-6, "rsw": 1e-4, "euler": 1e-4,
                  "boussinesq": 1e-4}


@pytest.mark.parametrize("case", ["islands", "periodic", "helmholtz"])
def test_fp32_model_poisson_reaches_fp64_accuracy(case):
    g = load("poisson.npz")
    nx, ny, xper = (int(v) for v in g[case + "/params"])
    helm = float(g[case + "/maindiag"]) != 0
    m = _model("qg" if helm else "eulerpsi", nx, ny, g[case + "/msk"],
               xperiodic=bool(xper), f0=float(g[case + "/f0"]), precision="fp32")
    solver = m.mesh.qg_helmholtz if helm else m.mesh.poisson_vertices
    x = g[case + "/x0"].copy()
    solver.solve(g[case + "/b"], x)
    assert rel_l2(x, g[case + "/x"]) <= SOLVE_TOL, rel_l2(x, g[case + "/x"])


@pytest.mark.parametrize("kind,integrator",
                         [("eulerpsi", "rk3"), ("rsw", "rk3"), ("qg", "rk3"),
                          ("eulerpsi", "LFRA"), ("rsw", "LFRA"), ("euler", "rk3"),
                          ("boussinesq", "rk3")])
def test_fp32_model_vs_fp64_oracle(kind, integrator):
    if kind == "euler":
        case = wl.euler_case(n=128, ny=96, seed=5, nislands=3)
    elif kind == "boussinesq":
        case = wl.boussinesq_case(n=128, ny=96, seed=6, nislands=3)
    elif kind == "eulerpsi":
        case = wl.eulerpsi_case(n=128, ny=96, seed=5, nislands=3)
    elif kind == "rsw":
        case = wl.rsw_case(n=128, ny=96, seed=6, nislands=3)
    else:
        case = wl.qg_case(n=128, ny=128, seed=7, nislands=4)
    om = _oracle_like(case, kind, integrator=integrator)
    kw = dict(xperiodic=case.get("xperiodic", False), Lx=case["Lx"], Ly=case["Ly"],
              tend=1e300, maxite=10 ** 9, precision="fp32", integrator=integrator)
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
    for _ in range(5):
        om.run_steps(1)
        m.advance(1)
    m.sync()
    worst = compare(m, lambda k: om.s.get(k), FP32_STATE_TOL[kind])
    print(f"FP32 {kind} {integrator} rel L2 after 5 steps:",
          {k: f"{v:.2e}" for k, v in worst.items()})


@pytest.mark.parametrize("kind", ["eulerpsi", "rsw"])
def test_lfra_restart_is_euler_forward(kind):
    """LFRA's first step is taken at ite == 0 (integrators.py:33): resetting
    the time line to ite = 0 restarts with an Euler-forward step, whatever the
    stored previous state; the leap-frog steps that follow match the oracle
    restarted from the same state."""
    case = (wl.eulerpsi_case(n=64, ny=48, seed=3, nislands=2) if kind == "eulerpsi"
            else wl.rsw_case(n=64, ny=48, seed=4, nislands=2))
    kw = dict(xperiodic=case.get("xperiodic", False), Lx=case["Lx"], Ly=case["Ly"],
              tend=1e300, maxite=10 ** 9, integrator="LFRA", cfl=0.4)
    for k in ("f0", "g", "H", "beta"):
        if k in case:
            kw[k] = case[k]
    m = _model(kind, case["nx"], case["ny"], case["msk"], **kw)
    s = m.state
    for k, v in case["fields"].items():
        getattr(s, k)[:] = v
    m.integrator.diag(s)
    m.advance(3)
    m.sync()
    # restart from the state reached: a fresh oracle (ite = 0) from it
    om = _oracle_like(case, kind, integrator="LFRA", cfl=0.4)
    for k in om.prog:
        v = getattr(m.state, k.split(".")[0])
        om.s[k][:] = getattr(v, k.split(".")[1]) if "." in k else v
    om.diag()
    m.time.ite = 0
    m.time.t = 0.0
    for _ in range(3):
        om.run_steps(1)
        m.advance(1)
    m.sync()
    compare(m, lambda k: om.s.get(k), STEP_TOL)


# ------------------------------------------------------------ ensembles ----
def _ensemble(members, precision="fp64", kind="eulerpsi", integrator="rk3"):
    p = f2d.Param()
    p.model = kind
    p.integrator = integrator
    p.cfl = 0.8
    p.tend = 1e300
    p.maxite = 10 ** 9
    p.precision = precision
    if kind == "qg":
        p.f0, p.beta = members[0]["f0"], members[0]["beta"]
    e = f2d.Ensemble(p, [(c["nx"], c["ny"]) for c in members],
                     [c["msk"] for c in members])
    for b, c in enumerate(members):
        for k, v in c["fields"].items():
            e.set_field(b, k, v)
        if "f" in c:
            e.set_field(b, "f", c["f"])
    e.diag()
    return e


@pytest.mark.parametrize("precision,integrator",
                         [("fp64", "rk3"), ("fp32", "rk3"), ("fp64", "enrk3"),
                          ("fp64", "LFRA"), ("fp32", "LFRA")])
def test_ensemble_members_match_single_models(precision, integrator):
    """Every member equals the same case run alone (same device code, same
    per-member reductions): FP64 to the step tolerance; FP32 to 1e-6, since
    the batched and the single-model stage kernels are separate
    instantiations whose multiply-adds the compiler may contract into FMAs
    differently, and FP32 rounding differences grow through the steps."""
    tol = STEP_TOL if precision == "fp64" else 1e-6
    members = [wl.eulerpsi_case(n=64, ny=48, seed=11, nislands=2),
               wl.eulerpsi_case(n=96, ny=96, seed=12, nislands=0),
               wl.eulerpsi_case(n=40, ny=72, seed=13, nislands=3)]
    e = _ensemble(members, precision, integrator=integrator)
    e.run(4)
    e.sync()
    for b, c in enumerate(members):
        m = _model("eulerpsi", c["nx"], c["ny"], c["msk"], cfl=0.8, tend=1e300,
                   maxite=10 ** 9, precision=precision, integrator=integrator)
        m.state.omega[:] = c["fields"]["omega"]
        m.integrator.diag(m.state)
        m.advance(4)
        m.sync()
        for k in ("omega", "psi", "U.x", "U.y"):
            a = e.get_field(b, k)
            r = getattr(m.state, k.split(".")[0])
            r = getattr(r, k.split(".")[1]) if "." in k else r
            assert rel_l2(a, r) <= tol, (b, k, rel_l2(a, r))
        t, dt, ite = e.time(b)
        assert ite == 4 and abs(t - m.time.t) <= 1e-12 * t


def test_autotune_ensemble_keeps_results():
    """The autotuner changes the multigrid schedule, not the solution: the
    tuned FP32 ensemble matches an untuned one to the FP32 tolerance."""
    members = [wl.eulerpsi_case(n=64, ny=48, seed=31, nislands=2),
               wl.eulerpsi_case(n=128, ny=96, seed=32, nislands=1)]
    e1 = _ensemble(members, "fp32")
    e1.run(3)
    e1.sync()
    e2 = _ensemble(members, "fp32")
    cfg = e2.autotune(reps=1)
    assert cfg["tile_rows"] in (32, 64) and cfg["sweeps"] in (1, 2)
    assert cfg["tol_in"] in (1e-8, 1e-7, 1e-6, 1e-5, 1e-4) and cfg["ms_per_solve"] > 0
    e2.run(3)
    e2.sync()
    for b in range(len(members)):
        for k in ("omega", "psi"):
            assert rel_l2(e2.get_field(b, k), e1.get_field(b, k)) <= 1e-6, (b, k)


@pytest.mark.parametrize("kind", ["qg", "qgrsw"])
def test_autotune_model_vs_oracle(kind):
    """A tuned FP64 model still matches the oracle at the step tolerance."""
    if kind == "qg":
        case = wl.qg_case(n=96, ny=96, seed=33, nislands=3)
    else:
        case = wl.rsw_case(n=96, ny=80, seed=34, nislands=2, xperiodic=False, f0=10.0)
        z = np.zeros_like(case["fields"]["h"])
        case["fields"] = {"u.x": z, "u.y": z.copy(), "h": case["fields"]["h"]}
    om = _oracle_like(case, kind, cfl=0.5)
    if kind == "qgrsw":
        O.qg_projection(om.mesh, om.s["u.x"], om.s["u.y"], om.s["h"], om.s["pv"],
                        om.s["psi"])
        om.diag()
    kw = dict(Lx=case["Lx"], Ly=case["Ly"], tend=1e300, maxite=10 ** 9, cfl=0.5)
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
    if kind == "qgrsw":
        m.qg_projection()
    m.integrator.diag(m.state)
    cfg = m.autotune(reps=1)
    assert cfg["tile_rows"] in (32, 64) and cfg["sweeps"] in (1, 2)
    for _ in range(3):
        om.run_steps(1)
        m.advance(1)
        compare(m, lambda k: om.s.get(k), STEP_TOL)
    m.sync()


def test_ensemble_fields_all_members_roundtrip():
    """f2d_ensemble_fields_set/get (all members, packed layout) agree with
    the per-member calls, FP64 and FP32 arenas."""
    members = [wl.eulerpsi_case(n=40, ny=24, seed=41, nislands=1),
               wl.eulerpsi_case(n=72, ny=56, seed=42, nislands=2),
               wl.eulerpsi_case(n=33, ny=47, seed=43, nislands=0)]
    for prec in ("fp64", "fp32"):
        e = _ensemble(members, prec)
        got = e.get_fields("omega")
        for b, c in enumerate(members):
            np.testing.assert_array_equal(got[b], e.get_field(b, "omega"))
        rng = np.random.default_rng(5)
        new = [rng.standard_normal(e.shape(b)) for b in range(len(members))]
        e.set_fields("omega", new)
        for b in range(len(members)):
            ref = new[b] if prec == "fp64" else new[b].astype(np.float32)
            np.testing.assert_array_equal(e.get_field(b, "omega"), ref)
        psi = e.get_fields("psi")
        for b in range(len(members)):
            np.testing.assert_array_equal(psi[b], e.get_field(b, "psi"))


def test_ensemble_fields_pinned():
    """The packed all-members I/O with pinned host buffers (the bench's
    end-to-end path) gives the pageable path's result."""
    import ctypes
    members = [wl.eulerpsi_case(n=40, ny=24, seed=41, nislands=1),
               wl.eulerpsi_case(n=72, ny=56, seed=42, nislands=2)]
    for prec in ("fp64", "fp32"):
        e = _ensemble(members, prec)
        n = e.packed_size()
        pinned = torch.empty(n, dtype=torch.float64, pin_memory=True)
        pageable = np.zeros(n)
        L = _lib.lib()
        assert L.f2d_ensemble_fields_get(e._h, b"omega", ctypes.c_void_p(pinned.data_ptr()),
                                         0) == 0
        assert L.f2d_ensemble_fields_get(e._h, b"omega", pageable.ctypes.data, 0) == 0
        np.testing.assert_array_equal(pinned.numpy(), pageable)
        rng = np.random.default_rng(9)
        new = rng.standard_normal(n)
        pinned.copy_(torch.from_numpy(new))
        assert L.f2d_ensemble_fields_set(e._h, b"omega", ctypes.c_void_p(pinned.data_ptr()),
                                         0) == 0
        back = np.zeros(n)
        assert L.f2d_ensemble_fields_get(e._h, b"omega", back.ctypes.data, 0) == 0
        ref = new if prec == "fp64" else new.astype(np.float32).astype(np.float64)
        # the packed layout covers every member's NY x NX array; compare all
        np.testing.assert_array_equal(back, ref)


def test_field_io_pinned():
    """f2d_field_set/get with pinned host memory (the bench's end-to-end
    path) give the pageable path's results, FP64 and FP32 models, an
    FP64-only field (psi) included."""
    import ctypes
    case = wl.eulerpsi_case(n=48, ny=40, seed=3, nislands=1)
    for prec in ("fp64", "fp32"):
        m = _model("eulerpsi", 48, 40, case["msk"], precision=prec)
        m.state.omega[:] = case["fields"]["omega"]
        m.integrator.diag(m.state)
        m.sync()
        L = _lib.lib()
        shape = m.mesh.shape
        for name in (b"omega", b"psi"):
            pinned = torch.empty(shape, dtype=torch.float64, pin_memory=True)
            pageable = np.zeros(shape)
            assert L.f2d_field_get(m._h, name, ctypes.c_void_p(pinned.data_ptr())) == 0
            assert L.f2d_field_get(m._h, name, pageable.ctypes.data) == 0
            np.testing.assert_array_equal(pinned.numpy(), pageable)
        new = np.random.default_rng(4).standard_normal(shape)
        pinned = torch.from_numpy(new.copy()).pin_memory()
        assert L.f2d_field_set(m._h, b"omega", ctypes.c_void_p(pinned.data_ptr())) == 0
        back = np.zeros(shape)
        assert L.f2d_field_get(m._h, b"omega", back.ctypes.data) == 0
        ref = new if prec == "fp64" else new.astype(np.float32).astype(np.float64)
        np.testing.assert_array_equal(back, ref)


def test_ensemble_vs_oracle():
    members = [wl.eulerpsi_case(n=48, ny=40, seed=21, nislands=2),
               wl.eulerpsi_case(n=72, ny=64, seed=22, nislands=1)]
    e = _ensemble(members, "fp64")
    e.run(3)
    e.sync()
    for b, c in enumerate(members):
        om = _oracle_like(c, "eulerpsi")
        om.p.cfl = 0.8
        om.dt = 0.01
        om.diag()
        om.run_steps(3)
        for k in ("omega", "psi"):
            assert rel_l2(e.get_field(b, k), om.s[k]) <= STEP_TOL
