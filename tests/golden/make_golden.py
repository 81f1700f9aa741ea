"""Generate the golden fixtures under tests/golden/ by running the reference.

Usage (needs the reference source tree, see ``refstubs.py``)::

    F2D_REFERENCE_SRC=<reference checkout>/src python tests/golden/make_golden.py

Each fixture is a compressed ``.npz`` holding the inputs and the outputs of
the unmodified reference code (``src/fluids2d``) on small seeded cases:

* ``mesh.npz``      - masks, slip coefficients, stencil orders and the
                      fluid-point index ``G`` for several masks
                      (``meshes.py:77-104, 146-186``; ``noslip.py:4-36``;
                      ``elliptic.py:102-111, 198-203``);
* ``sweeps.npz``    - the flat-index kernels ``compflux``, ``vortexforce``
                      and ``innerproduct`` for all four flux methods
                      (``weno.py:346-436``);
* ``poisson.npz``   - ``Poisson2D("v")`` solves with and without the
                      Helmholtz diagonal (``elliptic.py:71-87, 114-195``);
* ``model_*.npz``   - whole time steps of eulerpsi, rsw and qg driven the
                      way ``Model.run`` drives them (``model.py:45-51``):
                      ``set_dt`` then ``step(1)``, states saved every step.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from refstubs import load_reference  # noqa: E402
from forcings import BUILDERS as FORCINGS  # noqa: E402
from fluids2d_gb300 import workloads as wl  # noqa: E402

fd = load_reference()
from fluids2d import weno, elliptic  # noqa: E402


def make_param(model, nx, ny, **kw):
    p = fd.Param()
    p.model = model
    p.nx = nx
    p.ny = ny
    for k, v in kw.items():
        setattr(p, k, v)
    return p


# ---------------------------------------------------------------- mesh ----
def mesh_cases():
    out = {}
    cases = []
    # (name, nx, ny, xperiodic, nislands, maxorder, noslip, random)
    cases.append(("closed", 20, 16, False, 0, 6, None, False))
    cases.append(("islands", 28, 22, False, 3, 6, None, False))
    cases.append(("periodic", 26, 20, True, 3, 6, None, False))
    cases.append(("order4", 28, 22, False, 3, 4, None, False))
    cases.append(("order2", 28, 22, True, 3, 2, None, False))
    cases.append(("noslip", 24, 18, False, 2, 6, True, False))
    cases.append(("noslip_lt", 24, 18, True, 2, 6, ["left", "top"], False))
    cases.append(("random", 30, 24, False, 0, 6, None, True))
    cases.append(("random_per", 30, 24, True, 0, 6, None, True))
    names = []
    for (name, nx, ny, xper, nisl, maxo, noslip, rnd) in cases:
        p = make_param("rsw", nx, ny, xperiodic=xper, maxorder=maxo,
                       noslip=noslip)
        m = fd.Model(p)
        mesh = m.mesh
        x, y = mesh.xy("c")
        if nisl:
            wl.carve_islands(mesh.msk, x, y, nisl, 0.08, 0.18, seed=len(names),
                             margin=0.15)
        if rnd:
            rng = np.random.default_rng(7 + len(names))
            hole = rng.uniform(size=mesh.msk.shape) < 0.25
            mesh.msk[hole] = 0
        # the pieces of Mesh.finalize that build masks, slip coefficients and
        # stencil orders (meshes.py:34-37); the LU factorisations are left out
        # because a random mask can isolate cells, which makes SuperLU fail
        mesh.set_masks()
        mesh.slipcoef = fd.meshes.get_slipcoef(p, mesh.msk)
        mesh.set_stencils(p.maxorder)
        pre = name + "/"
        out[pre + "msk"] = mesh.msk.copy()
        out[pre + "params"] = np.array([nx, ny, int(xper), maxo])
        out[pre + "noslip"] = np.array(repr(noslip))
        for k in ("mskx", "msky", "mskv"):
            out[pre + k] = getattr(mesh, k).copy()
        out[pre + "slipcoef"] = np.asarray(mesh.slipcoef).copy()
        for st in ("oc", "ov", "ok"):
            out[pre + st + "x"] = getattr(mesh, st).x.copy()
            out[pre + st + "y"] = getattr(mesh, st).y.copy()
        out[pre + "Gc"] = elliptic.get_Gindex(
            elliptic.get_msk_from_mesh(mesh, "c"))
        out[pre + "Gv"] = elliptic.get_Gindex(
            elliptic.get_msk_from_mesh(mesh, "v"))
        names.append(name)
    out["names"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "mesh.npz"), **out)
    print("mesh.npz", len(names), "cases")


# -------------------------------------------------------------- sweeps ----
def sweep_cases():
    out = {}
    nx, ny = 26, 20
    p = make_param("rsw", nx, ny, xperiodic=True)
    m = fd.Model(p)
    mesh = m.mesh
    x, y = mesh.xy("c")
    wl.carve_islands(mesh.msk, x, y, 2, 0.08, 0.16, seed=3, margin=0.15)
    mesh.finalize()
    rng = np.random.default_rng(11)
    shape = mesh.shape
    q = rng.normal(size=shape)
    # a smooth part so that all WENO branches (smooth and non-smooth) occur
    q += 3 * np.sin(6 * x) * np.cos(4 * y)
    U = rng.normal(size=shape)
    V = rng.normal(size=shape)
    out["msk"] = mesh.msk.copy()
    out["q"], out["U"], out["V"] = q, U, V
    for k in ("ocx", "ocy", "ovx", "ovy", "okx", "oky"):
        st = getattr(mesh, k[:2])
        out[k] = getattr(st, k[2]).copy()
    for method in ("weno", "upwind", "centered", "cweno"):
        for d, s, s2, sign in (("x", mesh.xshift, mesh.yshift, -1),
                               ("y", mesh.yshift, mesh.xshift, +1)):
            flx = np.zeros(shape)
            weno.compflux(flx, U, q, getattr(mesh.oc, d), s, method)
            out[f"compflux/{method}/{d}"] = flx
            du = np.zeros(shape)
            weno.vortexforce(du, V, q, getattr(mesh.ov, d), s, s2, sign,
                             method)
            out[f"vortexforce/{method}/{d}"] = du
            ke = rng.normal(size=shape) * 0.0 + 0.5  # accumulates in place
            out[f"innerproduct_in/{method}/{d}"] = ke.copy()
            weno.innerproduct(ke, U, q, getattr(mesh.ok, d), s, method)
            out[f"innerproduct/{method}/{d}"] = ke
    out["shifts"] = np.array([mesh.xshift, mesh.yshift])
    np.savez_compressed(os.path.join(HERE, "sweeps.npz"), **out)
    print("sweeps.npz")


# ------------------------------------------------------------- poisson ----
def poisson_cases():
    out = {}
    names = []
    for (name, nx, ny, xper, nisl, model, f0) in (
            ("closed", 32, 24, False, 0, "eulerpsi", 10.0),
            ("islands", 36, 30, False, 3, "eulerpsi", 10.0),
            ("periodic", 32, 28, True, 2, "eulerpsi", 10.0),
            ("helmholtz", 36, 30, False, 3, "qg", 50.0),
            ("helmholtz_per", 32, 28, True, 2, "qg", 50.0)):
        p = make_param(model, nx, ny, xperiodic=xper, f0=f0)
        m = fd.Model(p)
        mesh = m.mesh
        x, y = mesh.xy("c")
        if nisl:
            wl.carve_islands(mesh.msk, x, y, nisl, 0.06, 0.14,
                             seed=20 + len(names), margin=0.15)
        mesh.finalize()
        rng = np.random.default_rng(30 + len(names))
        b = rng.normal(size=mesh.shape) * mesh.mskv
        solver = mesh.qg_helmholtz if model == "qg" else mesh.poisson_vertices
        xsol = rng.normal(size=mesh.shape)  # non-fluid entries must survive
        x0 = xsol.copy()
        solver.solve(b, xsol)
        pre = name + "/"
        out[pre + "msk"] = mesh.msk.copy()
        out[pre + "params"] = np.array([nx, ny, int(xper)])
        out[pre + "f0"] = np.array(f0)
        out[pre + "maindiag"] = np.array(
            mesh.area * f0 ** 2 / (p.g * p.H) if model == "qg" else 0.0)
        out[pre + "b"] = b
        out[pre + "x0"] = x0
        out[pre + "x"] = xsol
        names.append(name)
    out["names"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "poisson.npz"), **out)
    print("poisson.npz", names)


# -------------------------------------------------------------- models ----
def run_model(case, nsteps, fname, cfl=None, extra=None, setup=None, forcing=None):
    kw = dict(xperiodic=case.get("xperiodic", False), Lx=case["Lx"],
              Ly=case["Ly"], tend=1e9, maxite=10 ** 9)
    for k in ("f0", "g", "H", "beta"):
        if k in case:
            kw[k] = case[k]
    if cfl is not None:
        kw["cfl"] = cfl
    if extra:
        kw.update(extra)
    p = make_param(case["model"], case["nx"], case["ny"], **kw)
    m = fd.Model(p)
    m.mesh.msk[:] = case["msk"]
    m.mesh.finalize()
    if "f" in case:
        m.mesh.f = case["f"].copy()
    for k, v in case["fields"].items():
        if "." in k:
            getattr(getattr(m.state, k.split(".")[0]), k.split(".")[1])[:] = v
        else:
            getattr(m.state, k)[:] = v
    if forcing is not None:
        # Model.add_forcing (model.py:121-123) with a forcing function of
        # tests/golden/forcings.py; the time line is attached to the mesh the
        # way the reference's experiment scripts do it
        m.mesh.time = m.time
        m.add_forcing(FORCINGS[forcing](m))
    pre = {}
    if setup is not None:
        # an initial-state operator of the reference (e.g. qg_projection);
        # the fixture's initial condition is the state it leaves, the state
        # it was applied to is kept as pre/<field>
        for name in setup.fields:
            v = getattr(m.state, name.split(".")[0])
            v = getattr(v, name.split(".")[1]) if "." in name else v
            pre[name] = v.copy()
        setup(m)
        case = dict(case)
        case["fields"] = {}
        for name in setup.fields:
            v = getattr(m.state, name.split(".")[0])
            v = getattr(v, name.split(".")[1]) if "." in name else v
            case["fields"][name] = v.copy()
    m.integrator.diag(m.state)

    out = {"msk": case["msk"].copy(), "model": np.array(case["model"]),
           "params": np.array([case["nx"], case["ny"],
                               int(kw["xperiodic"])]),
           "scalars": np.array([case["Lx"], case["Ly"], p.f0, p.beta, p.g,
                                p.H, p.cfl])}
    if "f" in case:
        out["f"] = case["f"].copy()
    if extra and "integrator" in extra:
        out["integrator"] = np.array(extra["integrator"])
    if extra and "RAgamma" in extra:
        out["RAgamma"] = np.array(float(extra["RAgamma"]))
    if extra and "tracer" in extra:
        out["tracer"] = np.array(extra["tracer"])
    if extra and "innerproduct" in extra:
        out["innerproduct"] = np.array(extra["innerproduct"])
    if forcing is not None:
        out["forcing"] = np.array(forcing)
    for k, v in case["fields"].items():
        out["ic/" + k] = v.copy()
    for k, v in pre.items():
        out["pre/" + k] = v

    def dump(prefix):
        for name in m.state._fields:
            v = getattr(m.state, name)
            if hasattr(v, "_fields"):
                out[f"{prefix}/{name}.x"] = v.x.copy()
                out[f"{prefix}/{name}.y"] = v.y.copy()
            else:
                out[f"{prefix}/{name}"] = v.copy()

    dump("step0")
    # one right-hand side evaluation on the initial state (rk3 stage 1 rhs)
    ds = m.integrator.scratch[0]
    m.integrator.rhs(m.state, ds)
    for name in ds._fields:
        v = getattr(ds, name)
        if hasattr(v, "_fields"):
            out[f"rhs0/{name}.x"] = v.x.copy()
            out[f"rhs0/{name}.y"] = v.y.copy()
        else:
            out[f"rhs0/{name}"] = v.copy()
    dts = []
    for k in range(1, nsteps + 1):
        m.set_dt()
        dts.append(m.time.dt)
        m.step(1)
        dump(f"step{k}")
    out["dt"] = np.array(dts)
    out["t"] = np.array(m.time.t)
    np.savez_compressed(os.path.join(HERE, fname), **out)
    print(fname, "steps", nsteps, "dt", dts[:3])


def model_cases():
    c = wl.eulerpsi_case(n=32, seed=1)
    run_model(c, 6, "model_eulerpsi.npz", cfl=0.8)
    c = wl.eulerpsi_case(n=40, ny=32, seed=2, nislands=2, nvortices=5,
                         radius=0.08)
    run_model(c, 5, "model_eulerpsi_islands.npz", cfl=0.8)
    c = wl.rsw_case(n=40, ny=32, seed=3, nislands=2)
    run_model(c, 5, "model_rsw.npz")
    c = wl.qg_case(n=40, ny=32, seed=4, nislands=3, kmin=2, kmax=8)
    run_model(c, 5, "model_qg.npz")


def euler_cases():
    """The euler model (equations.py:9-24): momentum-pressure form with the
    Neumann cell-centred pressure projection (operators.py:114-119)."""
    c = wl.euler_case(n=40, ny=32, seed=5, nislands=2)
    run_model(c, 4, "model_euler.npz", cfl=0.5)
    c = wl.euler_case(n=40, ny=32, seed=6, nislands=2, xperiodic=True)
    run_model(c, 4, "model_euler_periodic.npz", cfl=0.5)


def boussinesq_cases():
    """The boussinesq model (equations.py:27-44): euler + buoyancy force
    (operators.py:152-153) + the flux divergence of the buoyancy b."""
    c = wl.boussinesq_case(n=40, ny=32, seed=8, nislands=2)
    run_model(c, 4, "model_boussinesq.npz", cfl=0.5)
    c = wl.boussinesq_case(n=40, ny=32, seed=9, nislands=1, xperiodic=True)
    run_model(c, 4, "model_boussinesq_periodic.npz", cfl=0.5)
    c = wl.boussinesq_case(n=40, ny=32, seed=10, nislands=2)
    run_model(c, 4, "model_boussinesq_lfra.npz", cfl=0.4,
              extra={"integrator": "LFRA"})


def tracer_cases():
    """A passive tracer appended to each model's equations
    (addtracerequation, equations.py:217-226) in closed basins (the
    reference does not fill the tracer tendency's x-periodic halo)."""
    c = wl.add_tracer(wl.eulerpsi_case(n=40, ny=32, seed=2, nislands=2,
                                       nvortices=5, radius=0.08), seed=1)
    run_model(c, 4, "model_eulerpsi_tracer.npz", cfl=0.8, extra={"tracer": "q"})
    c = wl.add_tracer(wl.qg_case(n=40, ny=32, seed=4, nislands=3, kmin=2,
                                 kmax=8), name="c", seed=2)
    run_model(c, 4, "model_qg_tracer_lfra.npz", cfl=0.4,
              extra={"tracer": "c", "integrator": "LFRA"})
    c = wl.add_tracer(wl.rsw_case(n=40, ny=32, seed=3, nislands=2,
                                  xperiodic=False), seed=3)
    run_model(c, 4, "model_rsw_tracer.npz", extra={"tracer": "q"})
    c = wl.add_tracer(wl.boussinesq_case(n=40, ny=32, seed=8, nislands=2),
                      name="s", seed=4)
    run_model(c, 4, "model_boussinesq_tracer.npz", cfl=0.5,
              extra={"tracer": "s"})
    # qgrsw with a tracer: the tracer advected by the projected flow
    from fluids2d.operators import qg_projection

    def project(m):
        s = m.state
        qg_projection(m.mesh, s.u, s.h, s.pv, s.psi)
    project.fields = ("u.x", "u.y", "h", "pv", "psi", "q")
    c = wl.rsw_case(n=40, ny=32, seed=11, nislands=2, xperiodic=False, f0=10.0)
    c["model"] = "qgrsw"
    c["fields"] = {"u.x": np.zeros_like(c["fields"]["h"]),
                   "u.y": np.zeros_like(c["fields"]["h"]), "h": c["fields"]["h"]}
    c = wl.add_tracer(c, seed=5)
    run_model(c, 4, "model_qgrsw_tracer.npz", cfl=0.5, extra={"tracer": "q"},
              setup=project)


def qgrsw_cases():
    """The qgrsw model (equations.py:104-135): the RSW tendency projected on
    the QG manifold each stage (qg_projection, operators.py:176-211). The
    initial state is h of a shallow-water bump projected by the reference's
    qg_projection (anomaly=False), as in its geostrophic-adjustment
    experiment; the reference writes nan into cells without a wet vertex."""
    from fluids2d.operators import qg_projection

    def project(m):
        s = m.state
        qg_projection(m.mesh, s.u, s.h, s.pv, s.psi)
    project.fields = ("u.x", "u.y", "h", "pv", "psi")

    for xper, seed, fname, extra in ((False, 3, "model_qgrsw.npz", None),
                                     (True, 5, "model_qgrsw_periodic.npz", None),
                                     (False, 7, "model_qgrsw_lfra.npz",
                                      {"integrator": "LFRA"})):
        c = wl.rsw_case(n=40, ny=32, seed=seed, nislands=2, xperiodic=xper, f0=10.0)
        c["model"] = "qgrsw"
        c["fields"] = {"u.x": np.zeros_like(c["fields"]["h"]),
                       "u.y": np.zeros_like(c["fields"]["h"]),
                       "h": c["fields"]["h"]}
        run_model(c, 4, fname, cfl=0.5, extra=extra, setup=project)


def bulk_cases():
    """Bulk diagnostics (diagnostics.py:39-57) along a trajectory: the
    reference's Bulk.__call__ after every step (it records every third
    iteration). The NetCDF file it would create is skipped (netCDF4 is
    absent): get_number_of_records is made to report an existing file."""
    from fluids2d import diagnostics as rdiag
    rdiag.get_number_of_records = lambda ncfile: 1
    cases = ((wl.rsw_case(n=40, ny=32, seed=3, nislands=2), "bulk_rsw.npz", None),
             (wl.euler_case(n=40, ny=32, seed=5, nislands=2), "bulk_euler.npz", 0.5))
    for case, fname, cfl in cases:
        kw = dict(xperiodic=case.get("xperiodic", False), Lx=case["Lx"],
                  Ly=case["Ly"], tend=1e9, maxite=10 ** 9)
        for k in ("f0", "g", "H", "beta"):
            if k in case:
                kw[k] = case[k]
        if cfl is not None:
            kw["cfl"] = cfl
        p = make_param(case["model"], case["nx"], case["ny"], **kw)
        m = fd.Model(p)
        m.mesh.msk[:] = case["msk"]
        m.mesh.finalize()
        for k, v in case["fields"].items():
            if "." in k:
                getattr(getattr(m.state, k.split(".")[0]), k.split(".")[1])[:] = v
            else:
                getattr(m.state, k)[:] = v
        m.integrator.diag(m.state)
        b = rdiag.Bulk(m)
        b()
        dts = []
        for _ in range(7):
            m.set_dt()
            dts.append(m.time.dt)
            m.step(1)
            b()
        out = {"msk": case["msk"].copy(), "model": np.array(case["model"]),
               "params": np.array([case["nx"], case["ny"], int(kw["xperiodic"])]),
               "scalars": np.array([case["Lx"], case["Ly"], p.f0, p.beta, p.g,
                                    p.H, p.cfl]),
               "dt": np.array(dts),
               "bulk": np.stack([x[:b.kt] for x in b.data], axis=1)}
        for k, v in case["fields"].items():
            out["ic/" + k] = v.copy()
        np.savez_compressed(os.path.join(HERE, fname), **out)
        print(fname, "records", b.kt)


def integrator_cases():
    """The reference's other Runge-Kutta integrators (integrators.py:116-155)."""
    c = wl.eulerpsi_case(n=40, ny=32, seed=2, nislands=2, nvortices=5,
                         radius=0.08)
    run_model(c, 4, "model_eulerpsi_ef.npz", cfl=0.4, extra={"integrator": "ef"})
    run_model(c, 4, "model_eulerpsi_enrk3.npz", cfl=0.8,
              extra={"integrator": "enrk3"})
    c = wl.rsw_case(n=40, ny=32, seed=3, nislands=2)
    run_model(c, 4, "model_rsw_enrk3.npz", extra={"integrator": "enrk3"})
    lfra_cases()


def lfra_cases():
    """Leap-frog with the Robert-Asselin filter (integrators.py:20-55): an
    Euler-forward first step, then leap-frog steps."""
    c = wl.eulerpsi_case(n=40, ny=32, seed=2, nislands=2, nvortices=5,
                         radius=0.08)
    run_model(c, 6, "model_eulerpsi_lfra.npz", cfl=0.4,
              extra={"integrator": "LFRA"})
    c = wl.qg_case(n=40, ny=32, seed=4, nislands=3, kmin=2, kmax=8)
    run_model(c, 5, "model_qg_lfra.npz", cfl=0.4,
              extra={"integrator": "LFRA", "RAgamma": 0.2})
    c = wl.rsw_case(n=40, ny=32, seed=3, nislands=2)
    run_model(c, 6, "model_rsw_lfra.npz", cfl=0.4, extra={"integrator": "LFRA"})
    c = wl.euler_case(n=40, ny=32, seed=6, nislands=2, xperiodic=True)
    run_model(c, 5, "model_euler_lfra_periodic.npz", cfl=0.4,
              extra={"integrator": "LFRA"})


def forcing_cases():
    """Model.add_forcing (model.py:121-123, equations.py:229-238) with the
    forcing functions of tests/golden/forcings.py."""
    c = wl.boussinesq_case(n=40, ny=32, seed=16, nislands=1)
    run_model(c, 4, "model_boussinesq_forced.npz", cfl=0.5, forcing="buoyancy_rows")
    c = wl.qg_case(n=40, ny=32, seed=17, nislands=2, kmin=2, kmax=8)
    run_model(c, 4, "model_qg_forced.npz", forcing="wind_curl")
    c = wl.euler_case(n=40, ny=32, seed=18, nislands=1)
    run_model(c, 4, "model_euler_forced_time.npz", cfl=0.5, forcing="wave_maker")
    c = wl.rsw_case(n=40, ny=32, seed=19, nislands=2)
    run_model(c, 4, "model_rsw_forced_periodic.npz", forcing="periodic_mass_source")
    c = wl.euler_case(n=40, ny=32, seed=20, nislands=1)
    run_model(c, 5, "model_euler_forced_lfra.npz", cfl=0.4, forcing="wave_maker",
              extra={"integrator": "LFRA"})


def classic_cases():
    """innerproduct="classic" (operators.py:86-98): the 4-point kinetic
    energy of rsw, euler and boussinesq."""
    c = wl.rsw_case(n=40, ny=32, seed=13, nislands=2)
    run_model(c, 4, "model_rsw_classic.npz", extra={"innerproduct": "classic"})
    c = wl.euler_case(n=40, ny=32, seed=14, nislands=2, xperiodic=True)
    run_model(c, 4, "model_euler_classic_periodic.npz", cfl=0.5,
              extra={"innerproduct": "classic"})
    c = wl.boussinesq_case(n=40, ny=32, seed=15, nislands=1)
    run_model(c, 4, "model_boussinesq_classic.npz", cfl=0.5,
              extra={"innerproduct": "classic"})


if __name__ == "__main__":
    which = sys.argv[1:] or ["mesh", "sweeps", "poisson", "models", "integrators",
                             "euler", "boussinesq", "tracer", "qgrsw", "bulk"]
    if "lfra" in which:
        lfra_cases()
    if "classic" in which:
        classic_cases()
    if "forcing" in which:
        forcing_cases()
    if "boussinesq" in which:
        boussinesq_cases()
    if "tracer" in which:
        tracer_cases()
    if "qgrsw" in which:
        qgrsw_cases()
    if "bulk" in which:
        bulk_cases()
    if "mesh" in which:
        mesh_cases()
    if "sweeps" in which:
        sweep_cases()
    if "poisson" in which:
        poisson_cases()
    if "models" in which:
        model_cases()
    if "integrators" in which:
        integrator_cases()
    if "euler" in which:
        euler_cases()
