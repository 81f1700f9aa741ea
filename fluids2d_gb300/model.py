"""Model, Mesh, State and Time: drop-in counterparts of the reference's
``fluids2d.Model`` (model.py), ``Mesh`` (meshes.py), state namedtuples
(states.py) and ``Time`` (timeline.py).

The state lives on the GPU. ``model.state`` is a namedtuple of host numpy
arrays with the reference's names and layout ((ny+6, nx+6) float64); it is
refreshed from the device when read and written back before the next GPU
operation, so user code that edits ``model.state.<var>`` in place (initial
conditions, callbacks) works as with the reference.
"""
from __future__ import annotations

import ctypes
import math
import signal
import time as _time
from collections import namedtuple

import numpy as np

from . import _lib
from . import io as _io
from ._lib import check, lib, ptr
from .param import Param

# states.py:7-17 for the models of the GPU path
MODEL_SPECS = {
    "eulerpsi": (("omega", "U", "psi", "vomega", "flx"), ("omega",)),
    "euler": (("u", "U", "omega", "ke", "p", "div", "flx"), ("u",)),
    "boussinesq": (("b", "u", "U", "omega", "ke", "p", "div", "flx"), ("b", "u")),
    "rsw": (("u", "h", "U", "omega", "ke", "p", "flx", "pv"), ("u", "h")),
    "qg": (("pv", "U", "h", "flx", "work", "psi"), ("pv",)),
    "qgrsw": (("u", "h", "U", "omega", "ke", "p", "flx", "pv", "psi"), ("u", "h")),
}
VECTORS = ("u", "U", "flx", "v")
Vector = namedtuple("vector", ("x", "y"))


def has_tracer(param):
    tr = getattr(param, "tracer", None)
    return tr is not None and tr != "None"


def _specs(param):
    """states.py:22-34: with a tracer, the variables are the prognostic ones,
    the tracer, then the rest."""
    names, prog = MODEL_SPECS[param.model]
    if has_tracer(param):
        prog = prog + (param.tracer,)
        names = prog + names[len(prog) - 1:]
    return names, prog


def _allocate_state(param, shape):
    names, _ = _specs(param)
    State = namedtuple("state", names)
    content = {}
    for n in names:
        if n in VECTORS:
            content[n] = Vector(np.zeros(shape), np.zeros(shape))
        else:
            content[n] = np.zeros(shape)
    return State(**content)


def _flat_fields(state, tracer=None):
    """(device name, host array) pairs: vector fields become 'U.x', 'U.y';
    the tracer (named by param.tracer) is the device field 'tracer'."""
    out = []
    for name in state._fields:
        v = getattr(state, name)
        if isinstance(v, Vector):
            out.append((name + ".x", v.x))
            out.append((name + ".y", v.y))
        else:
            out.append(("tracer" if name == tracer else name, v))
    return out


class Time:
    """timeline.py:4-51; t, dt and ite are kept on the device."""

    def __init__(self, model):
        self._m = model
        p = model.param
        self.t0 = 0.0
        self.ite0 = 0

    def _get(self):
        t, dt, ite = ctypes.c_double(), ctypes.c_double(), ctypes.c_int64()
        check(lib().f2d_time_get(self._m._h, ctypes.byref(t), ctypes.byref(dt),
                                 ctypes.byref(ite)))
        return t.value, dt.value, ite.value

    def _set(self, t=None, dt=None, ite=None):
        t0, dt0, ite0 = self._get()
        check(lib().f2d_time_set(self._m._h, t0 if t is None else t,
                                 dt0 if dt is None else dt,
                                 ite0 if ite is None else ite))

    @property
    def t(self):
        return self._get()[0]

    @t.setter
    def t(self, v):
        self._set(t=float(v))

    @property
    def dt(self):
        return self._get()[1]

    @dt.setter
    def dt(self, v):
        self._set(dt=float(v))

    @property
    def ite(self):
        return self._get()[2]

    @ite.setter
    def ite(self, v):
        self._set(ite=int(v))

    @property
    def finished(self):
        t, _, ite = self._get()
        p = self._m.param
        return (t >= self.t0 + p.tend) or (ite >= self.ite0 + p.maxite)

    def tostring(self):
        return f"t={self.t:.2f}"


class _Solver:
    """Poisson2D facade: solve(b, x) writes the fluid points of x and applies
    the halo fill (elliptic.py:80-87)."""

    def __init__(self, model, which):
        self._m = model
        self.which = which
        self.last_iters = 0
        self.last_relres = 0.0

    def solve(self, b, x):
        b = np.ascontiguousarray(b, dtype=np.float64)
        xx = np.ascontiguousarray(x, dtype=np.float64)
        it, rr = ctypes.c_int(), ctypes.c_double()
        self._m._push()
        check(lib().f2d_poisson_solve(self._m._h, self.which, ptr(b), ptr(xx),
                                      ctypes.byref(it), ctypes.byref(rr)))
        self.last_iters, self.last_relres = it.value, rr.value
        if xx is not x:
            x[...] = xx
        return x


class Mesh:
    """meshes.py:7-111: geometry, masks and stencil orders (host copies),
    ``finalize()`` after editing ``msk``."""

    def __init__(self, model):
        self._m = model
        p = model.param
        self.param = p
        h = p.halowidth
        self.shape = (p.ny + 2 * h, p.nx + 2 * h)
        self.nx, self.ny = p.nx, p.ny
        self.dx = p.Lx / self.nx
        self.dy = p.Ly / self.ny
        self.area = self.dx * self.dy
        self.xshift = 1
        self.yshift = self.shape[-1]
        self.msk = np.zeros(self.shape, dtype="i1")
        xs = slice(None) if p.xperiodic else slice(h, -h)
        ys = slice(None) if p.yperiodic else slice(h, -h)
        self.msk[ys, xs] = 1
        self.hb = 0
        self._f = None
        self.poisson_vertices = _Solver(model, 0)
        if p.model in ("qg", "qgrsw", "rsw"):
            self.qg_helmholtz = _Solver(model, 1)
            self.qgcoef = p.f0 / +p.H
        self._derive()

    def _derive(self):
        d = _lib.mesh_build(self.param, self.msk)
        self.mskx, self.msky, self.mskv = d["mskx"], d["msky"], d["mskv"]
        self.slipcoef = d["slipcoef"]
        Stencil = namedtuple("stencil", ("x", "y"))
        self.oc = Stencil(d["ocx"], d["ocy"])
        self.ov = Stencil(d["ovx"], d["ovy"])
        self.ok = Stencil(d["okx"], d["oky"])
        self.G_vertices = d["gv"]

    def finalize(self):
        """Recompute everything derived from msk (meshes.py:34-52)."""
        m = np.ascontiguousarray(self.msk, dtype=np.int8)
        check(lib().f2d_model_set_mask(self._m._h, ptr(m)))
        self._derive()

    @property
    def f(self):
        return self._f

    @f.setter
    def f(self, value):
        """Vertex Coriolis term of the beta-plane (used by qg_inversion)."""
        a = np.ascontiguousarray(value, dtype=np.float64)
        check(lib().f2d_set_coriolis(self._m._h, ptr(a)))
        self._f = a

    def x(self, which):
        idx = np.arange(self.nx + 2 * self.param.halowidth) - self.param.halowidth
        shift = 0.5 if which in ["c", "y"] else 0.0
        return (idx + shift) * self.dx

    def y(self, which):
        idx = np.arange(self.ny + 2 * self.param.halowidth) - self.param.halowidth
        shift = 0.5 if which in ["c", "x"] else 0.0
        return (idx + shift) * self.dy

    def xy(self, which="c"):
        return np.meshgrid(self.x(which), self.y(which))

    def fill(self, variable):
        """Periodic halo copy on host arrays (meshes.py:106-143)."""
        if hasattr(variable, "_fields"):
            for v in variable:
                self.fill(v)
            return
        if self.param.xperiodic:
            n = self.param.halowidth
            variable[:, :n] = variable[:, -2 * n:-n]
            variable[:, -n:] = variable[:, n:2 * n]


class Integrator:
    """The integrator facade (integrators.py:9-79): RKIntegrator for rk3, ef
    and enrk3, LFRAintegrator for LFRA; the scratch states live on the
    device. ``rhs`` and ``diag`` are the pair of the reference's
    get_rhs_and_diag registry (equations.py:190-210) on the GPU."""

    def __init__(self, model):
        self._m = model

    @property
    def nstages(self):
        return 1 if self._m.param.integrator in ("ef", "LFRA") else 3

    def diag(self, state=None):
        m = self._m
        if state is not None and state is not m._state:
            raise ValueError("diag() acts on the model's own state")
        m._push()
        check(lib().f2d_diag(m._h))
        m._device_newer = True

    def rhs(self, state, ds):
        """rhs(s, ds) of equations.py:73-157 (with the tracer equation and
        the forcing terms): the tendency of the model's state (its
        diagnostics current, as after diag) computed on the GPU and written
        into the host arrays of ``ds``, a prognostic namedtuple (or any
        object with the prognostic variables as attributes, vectors with
        .x/.y) such as ``model.new_prognostic()`` returns."""
        m = self._m
        if state is not m._state:
            raise ValueError("rhs() acts on the model's own state")
        if m._forcings:
            # forcing functions of this state (and time) first
            f = m._static_term()
            for fn in m._forcings:
                fn(m.param, m.mesh, m.state, f)
            m._upload_forcing(f)
        m._push()
        check(lib().f2d_rhs(m._h))
        if m.param.model == "qgrsw":
            # the projection of the tendency leaves its PV and streamfunction
            # in s.pv and s.psi, as in the reference (equations.py:121)
            for name in ("pv", "psi"):
                check(lib().f2d_field_get(m._h, name.encode(), ptr(getattr(m._state, name))))
        _, prog = _specs(m.param)
        for name in prog:
            v = getattr(ds, name)
            if isinstance(v, tuple) and hasattr(v, "x"):
                targets = ((name + ".x", v.x), (name + ".y", v.y))
            else:
                targets = (("tracer" if name == m._tracer else name, v),)
            for dev, arr in targets:
                out = np.empty(m.mesh.shape)
                check(lib().f2d_field_get(m._h, ("rhs." + dev).encode(), ptr(out)))
                arr[...] = out

    def step(self, state=None, time=None):
        self._m.step(1)


class Model:
    """model.py:13-123 on the GPU."""

    def __init__(self, param: Param):
        param.check()
        self.param = param
        h = ctypes.c_void_p()
        s = _lib.params_struct(param)
        check(lib().f2d_model_create(ctypes.byref(s), None, ctypes.byref(h)))
        self._h = h
        self.mesh = Mesh(self)
        self._state = _allocate_state(param, self.mesh.shape)
        self._tracer = param.tracer if has_tracer(param) else None
        self._host_dirty = False
        self._device_newer = False
        self.integrator = Integrator(self)
        self.time = Time(self)
        self.callbacks = []
        self.diags = []
        self._forcings = []
        self._static_forcings = []
        self.stop = False
        self.io = _io.IO(param, self.mesh, None, self.time)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().f2d_model_destroy(h)
            except Exception:
                pass
            self._h = ctypes.c_void_p()

    # -- state synchronisation -----------------------------------------
    @property
    def state(self):
        self._pull()
        self._host_dirty = True  # the caller may edit the arrays in place
        return self._state

    def _pull(self):
        if not self._device_newer:
            return
        for name, arr in _flat_fields(self._state, self._tracer):
            if name.startswith("flx"):
                continue
            check(lib().f2d_field_get(self._h, name.encode(), ptr(arr)))
        self._device_newer = False

    def _push(self):
        if not self._host_dirty:
            return
        for name, arr in _flat_fields(self._state, self._tracer):
            if name.startswith("flx"):
                continue
            a = np.ascontiguousarray(arr, dtype=np.float64)
            check(lib().f2d_field_set(self._h, name.encode(), ptr(a)))
        self._host_dirty = False

    def _device_state_changed(self):
        """The device state was written by a library call (the adjoint
        rollouts) outside step/run: host arrays are refreshed on next use."""
        self._host_dirty = False
        self._device_newer = True

    # -- time stepping ---------------------------------------------------
    def step(self, nsteps=1):
        """model.py:67-69 (time.dt is the current device dt)."""
        if self._forcings:
            self._stepped_with_forcing(nsteps, with_dt=False)
            return
        self._push()
        check(lib().f2d_step(self._h, int(nsteps)))
        self._device_newer = True

    def qg_projection(self):
        """qg_projection(mesh, s.u, s.h, s.pv, s.psi) (operators.py:176-183,
        anomaly=False) on the model's state, on the GPU: the qgrsw initial
        state of the reference's geostrophic-adjustment set-up."""
        self._push()
        check(lib().f2d_qg_projection(self._h))
        self._device_newer = True

    def set_dt(self):
        """model.py:71-87 (computed on the device)."""
        self._push()
        check(lib().f2d_set_dt(self._h))

    def autotune(self, reps=3):
        """Pick the multigrid schedule (tile rows, sweeps per leg, inner
        tolerance) of the Poisson/Helmholtz solver by timing each
        candidate's solve of the current state on the GPU (f2d_autotune);
        the state is unchanged. Returns the chosen schedule."""
        self._push()
        th, nu = ctypes.c_int(), ctypes.c_int()
        tin, ms = ctypes.c_double(), ctypes.c_double()
        check(lib().f2d_autotune(self._h, int(reps), ctypes.byref(th), ctypes.byref(nu),
                                 ctypes.byref(tin), ctypes.byref(ms)))
        self._device_newer = True
        return {"tile_rows": th.value, "sweeps": nu.value, "tol_in": tin.value,
                "ms_per_solve": ms.value}

    def set_schedule(self, tile_rows, sweeps, tol_in=1e-6):
        """Set the multigrid schedule directly (tile rows 32/64, sweeps per
        leg 1/2, inner tolerance of the FP32 form), e.g. one an earlier
        autotune() returned (f2d_set_schedule)."""
        self._push()
        check(lib().f2d_set_schedule(self._h, int(tile_rows), int(sweeps), float(tol_in)))

    def advance(self, nsteps):
        """nsteps iterations of the run-loop body: set_dt then step(1)."""
        if self._forcings:
            self._stepped_with_forcing(nsteps, with_dt=True)
            return
        self._push()
        check(lib().f2d_run(self._h, int(nsteps)))
        self._device_newer = True

    def sync(self):
        check(lib().f2d_sync(self._h))

    def run(self):
        """model.py:29-59 without animation and NetCDF output."""
        self.stop = False

        def handler(sig, frame):
            print("\n hit ctrl-C, stopping", end="")
            self.stop = True

        try:
            old = signal.signal(signal.SIGINT, handler)
        except ValueError:  # not in the main thread
            old = None
        tic = _time.time()
        p = self.param
        try:
            self.save_to_file()
            while not self.time.finished and not self.stop:
                _, _, ite = self.time._get()
                left = self.time.ite0 + p.maxite - ite
                # with an infinite end time, the step count alone decides;
                # callbacks, diagnostics and history run at every iteration
                # they would see in the reference
                n = left if not math.isfinite(p.tend) or p.tend >= 1e300 else 1
                if self.callbacks or self.diags:
                    n = 1
                if p.nhis > 0:
                    n = min(n, p.nhis - ite % p.nhis)
                self.advance(max(1, min(n, left)))
                self.execute_callbacks()
                self.compute_diags()
                self.save_to_file()
            self.sync()
        finally:
            if old is not None:
                signal.signal(signal.SIGINT, old)
        toc = _time.time()
        self.print_perf(toc - tic)
        self.finalize()

    def save_to_file(self):
        """model.py:109-111 with timeline.py:46-51 (every nhis iterations and
        at the end)."""
        p = self.param
        if p.nhis == 0:
            return
        _, _, ite = self.time._get()
        if ite % p.nhis == 0 or self.time.finished:
            self.io.write(self)

    def finalize(self):
        """model.py:61-65, and the history file written out."""
        for d in self.diags:
            d.finalize()
        if self.param.nhis > 0:
            self.io.flush()

    def print_perf(self, elapsed):
        nite = self.time.ite - self.time.ite0
        if nite > 0:
            perf = elapsed / (self.mesh.nx * self.mesh.ny * nite)
            print(f"\nElapsed: {elapsed:.2f} s  perf: {perf:.2e} s/dof")

    def execute_callbacks(self):
        for func in self.callbacks:
            func(self.param, self.mesh, self.state, self.time)

    def compute_diags(self):
        for d in self.diags:
            d()

    def new_prognostic(self):
        """A zero prognostic namedtuple (states.py Prognostic): the shape of
        the integrator's scratch and of rhs()'s ds argument."""
        _, prog = _specs(self.param)
        Prog = namedtuple("prognostic", prog)
        shape = self.mesh.shape
        return Prog(**{n: Vector(np.zeros(shape), np.zeros(shape)) if n in VECTORS
                       else np.zeros(shape) for n in prog})

    def add_forcing(self, forcing, static=False):
        """Model.add_forcing (model.py:121-123): forcing(param, mesh, s, ds)
        adds its term to the tendency ds after the right-hand side in every
        stage (addforcingterm, equations.py:229-238); several forcings apply
        in the order they were added.

        On the GPU the forcing term is a field per prognostic variable added
        inside the stage kernels. The function is called with the current
        state and a zero ``ds`` to form that field, so it must add to ds, as
        the reference's forcing functions do.

        static=True: the term does not change with time or state; the
        function is called once here, and steps run at full speed (graphs).
        static=False (the reference's semantics for any function): the
        function is called before every stage with the stage's state (and
        ``mesh.time`` if attached), the field is uploaded and the stage runs
        alone (f2d_stage), which costs a host round trip per stage."""
        if static:
            self._static_forcings.append(forcing)
            self._upload_forcing(self._static_term())
        else:
            self._forcings.append(forcing)

    def _static_term(self):
        ds = self.new_prognostic()
        for f in self._static_forcings:
            f(self.param, self.mesh, self.state, ds)
        return ds

    def _upload_forcing(self, ds):
        for name, arr in _flat_fields(ds, self._tracer):
            a = np.ascontiguousarray(arr, dtype=np.float64)
            check(lib().f2d_forcing_set(self._h, name.encode(), ptr(a)))

    def _stepped_with_forcing(self, nsteps, with_dt):
        """Steps with time- or state-dependent forcing functions: each stage
        alone, its forcing field formed on the host just before it."""
        base = self._static_term() if self._static_forcings else None
        for _ in range(int(nsteps)):
            self._push()
            if with_dt:
                check(lib().f2d_set_dt(self._h))
            for k in range(1, self.integrator.nstages + 1):
                ds = self.new_prognostic() if base is None else \
                    type(base)(*[Vector(v.x.copy(), v.y.copy()) if isinstance(v, Vector)
                                 else v.copy() for v in base])
                state = self.state
                for f in self._forcings:
                    f(self.param, self.mesh, state, ds)
                self._push()
                self._upload_forcing(ds)
                check(lib().f2d_stage(self._h, k))
                self._device_newer = True

    def poisson_iterations(self):
        return self.stats()[0]

    def stats(self):
        """(Poisson iterations so far, kernels per step outside the Poisson
        loops, kernels per Poisson iteration)."""
        it, n, b = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        check(lib().f2d_stats(self._h, ctypes.byref(it), ctypes.byref(n),
                              ctypes.byref(b)))
        return it.value, n.value, b.value
