"""ORACLE - test infrastructure only. Never imported by the product path.

CPU restatement of the reference's time-stepping path (pvthinker/Fluids2d):
mesh masks and stencil orders, the flat-index flux sweeps (through the C
restatement in ``sweeps.c``), the staggered C-grid operators, the masked
5-point Poisson/Helmholtz operators (vertex Dirichlet and cell-centred
Neumann) solved with SuperLU, the eulerpsi, rsw, qg, euler, boussinesq and
qgrsw equation sets with the passive tracer, the rk3/ef/enrk3/LFRA
integrators, the CFL time step and the Bulk diagnostics. It serves three
purposes:

* the oracle the CUDA path is compared with in ``tests/`` and in
  ``__graft_entry__.smoke``;
* the CPU-baseline leg of ``bench.py`` (numba-equivalent sweeps threaded
  with OpenMP, numpy operators, SuperLU solves);
* a restatement pinned against the reference itself: ``tests/golden/`` holds
  outputs of the unmodified reference (run here with numba stubbed out) and
  ``tests/test_oracle_golden.py`` checks this module against them.

Each function cites the reference lines it follows. The numpy expressions
keep the reference's operand order so that results agree bit for bit where
the reference's own arithmetic is deterministic.
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np
import scipy.sparse as sparse
import scipy.sparse.linalg as splinalg

from . import build as _build

METHODS = {"weno": 0, "upwind": 1, "centered": 2, "cweno": 3}

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        bp = ctypes.POINTER(ctypes.c_int8)
        i64 = ctypes.c_int64
        for sfx in ("", "_py"):
            f = getattr(L, "oracle_compflux" + sfx)
            f.argtypes = [ctypes.c_int, dp, dp, dp, bp, i64, i64, i64]
            f.restype = None
            f = getattr(L, "oracle_vortexforce" + sfx)
            f.argtypes = [ctypes.c_int, dp, dp, dp, bp, i64, i64, ctypes.c_int,
                          i64, i64]
            f.restype = None
            f = getattr(L, "oracle_innerproduct" + sfx)
            f.argtypes = [ctypes.c_int, dp, dp, dp, bp, i64, i64, i64]
            f.restype = None
        L.oracle_set_order.argtypes = [bp, i64, i64, ctypes.c_int, bp]
        L.oracle_set_order.restype = None
        L.oracle_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _dp(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _bp(a):
    assert a.dtype == np.int8 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int8))


# ----------------------------------------------------------- sweeps ------
# weno.py:412-436. `pysq` selects pow(x,2) (Python-float semantics, matches a
# numba-less run of the reference bit for bit) or x*x (numba semantics).

def compflux(flx, U, q, o, s, method="weno", pysq=True):
    f = lib().oracle_compflux_py if pysq else lib().oracle_compflux
    f(METHODS[method], _dp(flx), _dp(U), _dp(q), _bp(o), s, 0, q.size)


def vortexforce(du, V, q, o, s, s2, sign, method="weno", pysq=True):
    f = lib().oracle_vortexforce_py if pysq else lib().oracle_vortexforce
    f(METHODS[method], _dp(du), _dp(V), _dp(q), _bp(o), s, s2, sign, 0,
      du.size)


def innerproduct(ke, U, q, o, s, method="weno", pysq=True):
    f = lib().oracle_innerproduct_py if pysq else lib().oracle_innerproduct
    f(METHODS[method], _dp(ke), _dp(U), _dp(q), _bp(o), s, 0, ke.size)


def set_order(msk, shift, maxorder):
    """meshes.py:146-186 (through the C restatement)."""
    m = np.ascontiguousarray(msk, dtype=np.int8)
    o = np.zeros(m.shape, dtype=np.int8)
    lib().oracle_set_order(_bp(m), m.size, shift, maxorder, _bp(o))
    return o


# ------------------------------------------------------------- param -----

class Param:
    """The reference's parameter defaults (param.py:11-59), as a plain bag."""

    def __init__(self, **kw):
        self.model = "euler"
        self.nx = 40
        self.ny = 40
        self.Lx = 1.0
        self.Ly = 1.0
        self.xperiodic = False
        self.yperiodic = False
        self.halowidth = 3
        self.noslip = None
        self.f0 = 10.0
        self.beta = 0.0
        self.g = 1
        self.H = 1
        self.tend = 1.0
        self.dt = 0.0
        self.maxite = 100
        self.dtmax = 9e99
        self.integrator = "rk3"
        self.RAgamma = 0.1
        self.tracer = None
        self.cfl = 0.9
        self.compflux = "weno"
        self.vortexforce = "weno"
        self.innerproduct = "weno"
        self.maxorder = 6
        for k, v in kw.items():
            setattr(self, k, v)


# -------------------------------------------------------------- mesh -----

def slipcoef(param, msk):
    """noslip.py:4-36."""
    coef = np.zeros(msk.shape)
    coef[:, :] += msk
    coef[:, 1:] += msk[:, :-1]
    coef[1:, :] += msk[:-1, :]
    coef[1:, 1:] += msk[:-1, :-1]
    free = lambda x: 1 * (x == 4)  # noqa: E731
    nos = lambda x: np.minimum(x, 1)  # noqa: E731
    if (param.noslip is None) or (param.noslip is False):
        return free(coef)
    if param.noslip is True:
        return nos(coef)
    out = free(coef)
    nh = param.halowidth
    if "left" in param.noslip:
        out[:, nh] = nos(coef[:, nh])
    if "right" in param.noslip:
        out[:, -nh] = nos(coef[:, -nh])
    if "bottom" in param.noslip:
        out[nh, :] = nos(coef[nh, :])
    if "top" in param.noslip:
        out[-nh, :] = nos(coef[-nh, :])
    return out


def gindex(msk):
    """elliptic.py:198-203: row-major index of fluid points, -1 elsewhere."""
    G = np.zeros(msk.shape, dtype="i")
    G[msk == 0] = -1
    G[msk == 1] = np.arange(int(np.sum(msk == 1)))
    return G


class Mesh:
    """meshes.py:7-111 without the plotting helpers."""

    def __init__(self, param):
        self.param = param
        h = param.halowidth
        self.shape = (param.ny + 2 * h, param.nx + 2 * h)
        self.nx, self.ny = param.nx, param.ny
        self.dx = param.Lx / self.nx
        self.dy = param.Ly / self.ny
        self.area = self.dx * self.dy
        self.xshift = 1
        self.yshift = self.shape[-1]
        self.msk = np.zeros(self.shape, dtype="i1")
        xs = slice(None) if param.xperiodic else slice(h, -h)
        ys = slice(None) if param.yperiodic else slice(h, -h)
        self.msk[ys, xs] = 1
        self.hb = 0
        self.f = None
        self.finalize()

    def finalize(self):
        p = self.param
        self.set_masks()
        self.slipcoef = slipcoef(p, self.msk)
        mo = p.maxorder
        self.ocx = set_order(self.msk, self.xshift, mo)
        self.ocy = set_order(self.msk, self.yshift, mo)
        mv = (1 * (self.slipcoef > 0)).astype(np.int8)
        self.ovx = set_order(mv, -self.xshift, mo)
        self.ovy = set_order(mv, -self.yshift, mo)
        self.ovx *= self.msky
        self.ovy *= self.mskx
        self.okx = set_order(self.mskx, -self.xshift, mo)
        self.oky = set_order(self.msky, -self.yshift, mo)
        self._solvers = {}
        if p.model in ("qg", "qgrsw", "rsw"):
            self.maindiag = self.area * p.f0 ** 2 / (p.g * p.H)
            self.qgcoef = p.f0 / +p.H

    # The reference factorises its operators inside finalize(); here the
    # factorisation is deferred to first use (rsw never solves).
    @property
    def poisson_vertices(self):
        if "v" not in self._solvers:
            self._solvers["v"] = Poisson2D(self, maindiag=0)
        return self._solvers["v"]

    @property
    def poisson_centers(self):
        """Poisson2D(mesh, "c"): Neumann cell-centred operator (singular; the
        reference factorises it anyway and SuperLU picks the constant)."""
        if "c" not in self._solvers:
            self._solvers["c"] = Poisson2D(self, maindiag=0, location="c")
        return self._solvers["c"]

    @property
    def qg_helmholtz(self):
        if "h" not in self._solvers:
            self._solvers["h"] = Poisson2D(self, maindiag=self.maindiag)
        return self._solvers["h"]

    def set_masks(self):
        msk = self.msk
        self.mskx = np.zeros(self.shape, dtype="i1")
        self.mskx[:, 1:] = msk[:, 1:] * msk[:, :-1]
        self.msky = np.zeros(self.shape, dtype="i1")
        self.msky[1:, :] = msk[1:, :] * msk[:-1, :]
        self.mskv = np.zeros(self.shape, dtype="i1")
        self.mskv[1:, 1:] = (msk[:-1, 1:] * msk[:-1, :-1]
                             * msk[1:, 1:] * msk[1:, :-1])

    def x(self, which="c"):
        """meshes.py:57-62: coordinates of the array columns."""
        idx = np.arange(self.nx + 2 * self.param.halowidth) - self.param.halowidth
        return (idx + (0.5 if which in ("c", "y") else 0.0)) * self.dx

    def y(self, which="c"):
        """meshes.py:63-68: coordinates of the array rows."""
        idx = np.arange(self.ny + 2 * self.param.halowidth) - self.param.halowidth
        return (idx + (0.5 if which in ("c", "x") else 0.0)) * self.dy

    def xy(self, which="c"):
        return np.meshgrid(self.x(which), self.y(which))

    def fill(self, a):
        """fill_halo_array, meshes.py:135-143."""
        if self.param.xperiodic:
            n = self.param.halowidth
            a[:, :n] = a[:, -2 * n:-n]
            a[:, -n:] = a[:, n:2 * n]


def vertex_msk(mesh, location="v"):
    """get_msk_from_mesh, elliptic.py:102-111: the vertex ("v") or cell ("c")
    mask with the periodic halo columns removed."""
    base = mesh.msk if location == "c" else mesh.mskv
    if not mesh.param.xperiodic:
        return base
    n = mesh.param.halowidth
    m = base * 1
    m[:, :n] = 0
    m[:, -n:] = 0
    return m


def laplacian(mesh, maindiag, location="v"):
    """Masked 5-point operator (get_Laplacian_sparse, elliptic.py:114-195):
    vertices with Dirichlet walls, or cell centres with Neumann walls (the
    diagonal is minus the sum of the present neighbours' couplings),
    assembled with numpy in the reference's entry order (per point: west,
    east, south, north, diagonal) so that SuperLU sees the same matrix."""
    G = gindex(vertex_msk(mesh, location))
    ny, nx = G.shape
    N = int(np.sum(G > -1))
    dx2 = mesh.dy / mesh.dx
    dy2 = mesh.dx / mesh.dy
    xper = mesh.param.xperiodic
    n1 = mesh.param.halowidth if xper else 0
    J, I = np.nonzero(G > -1)
    Ipt = G[J, I]
    west = np.where(I > n1, G[J, np.maximum(I - 1, 0)],
                    G[J, -n1 - 1] if xper else -1)
    east = np.where(I < nx - 1 - n1, G[J, np.minimum(I + 1, nx - 1)],
                    G[J, n1] if xper else -1)
    south = np.where(J > 0, G[np.maximum(J - 1, 0), I], -1)
    north = np.where(J < ny - 1, G[np.minimum(J + 1, ny - 1), I], -1)
    if location == "v":
        diag = np.full(N, -2 * (dx2 + dy2) - maindiag)
    else:
        # sum_extra_diag accumulated in the reference's order
        sed = np.zeros(N)
        for nb, c in ((west, dx2), (east, dx2), (south, dy2), (north, dy2)):
            sed = np.where(nb > -1, sed + c, sed)
        diag = -sed - maindiag
    cols = np.stack([west, east, south, north, Ipt], axis=1)
    vals = np.stack([np.full(N, dx2), np.full(N, dx2), np.full(N, dy2),
                     np.full(N, dy2), diag], axis=1)
    valid = cols > -1
    rows = np.repeat(Ipt[:, None], 5, axis=1)
    cnt = int(valid.sum())
    data = np.zeros(5 * N)
    row = np.zeros(5 * N, dtype="i")
    col = np.zeros(5 * N, dtype="i")
    data[:cnt] = vals[valid]
    row[:cnt] = rows[valid]
    col[:cnt] = cols[valid]
    A = sparse.coo_matrix((data, (row, col)), shape=(N, N))
    return A.tocsc(), G


class Poisson2D:
    """Poisson2D "v" (elliptic.py:71-87): LU factorisation once, then
    back-substitution; only fluid points of x are written, then halo fill."""

    def __init__(self, mesh, maindiag=0, location="v"):
        self.mesh = mesh
        self.A, self.G = laplacian(mesh, maindiag, location)
        self.lu = splinalg.splu(self.A)

    def solve(self, b, x):
        sel = self.G > -1
        x[sel] = self.lu.solve(b[sel])
        self.mesh.fill(x)
        return x


# --------------------------------------------------------- operators -----

def div(mesh, Ux, Uy, delta):
    """operators.py:104-107."""
    delta[:, :-1] = -np.diff(Ux, axis=1)
    delta[:-1, :] -= np.diff(Uy, axis=0)
    delta *= mesh.msk


def divflux(p, mesh, fx, fy, q, Ux, Uy, dq, pysq):
    """operators.py:21-29."""
    compflux(fx, Ux, q, mesh.ocx, mesh.xshift, p.compflux, pysq)
    compflux(fy, Uy, q, mesh.ocy, mesh.yshift, p.compflux, pysq)
    div(mesh, fx, fy, dq)


def addvortexforce(p, mesh, Ux, Uy, omega, dux, duy, pysq):
    """operators.py:6-15."""
    vortexforce(dux, Uy, omega, mesh.ovy, mesh.yshift, mesh.xshift, +1,
                p.vortexforce, pysq)
    vortexforce(duy, Ux, omega, mesh.ovx, mesh.xshift, mesh.yshift, -1,
                p.vortexforce, pysq)


def addcoriolis(p, mesh, Ux, Uy, dux, duy):
    """operators.py:32-39."""
    f = p.f0 * mesh.area * 0.25
    dux[:-1, 1:-1] += f * (Uy[:-1, :-2] + Uy[1:, :-2] +
                           Uy[:-1, 1:-1] + Uy[1:, 1:-1])
    duy[1:-1, :-1] -= f * (Ux[:-2, :-1] + Ux[:-2, 1:] +
                           Ux[1:-1, :-1] + Ux[1:-1, 1:])


def addgrad(mesh, phi, dux, duy):
    """operators.py:49-53."""
    dux[:, 1:] -= np.diff(phi, axis=1) * mesh.mskx[:, 1:]
    duy[1:, :] -= np.diff(phi, axis=0) * mesh.msky[1:, :]


def addbuoyancy(mesh, b, duy):
    """operators.py:152-153."""
    duy[1:, :] += (0.5 * mesh.dy) * (b[1:, :] + b[:-1, :]) * mesh.msky[1:, :]


def sharp(mesh, ux, uy, Ux, Uy):
    """operators.py:59-62."""
    Ux[:] = ux * (1 / mesh.dx ** 2)
    Uy[:] = uy * (1 / mesh.dy ** 2)


def compute_vorticity(mesh, ux, uy, omega):
    """operators.py:67-72, 77."""
    omega[1:, :] = -np.diff(ux, axis=0)
    omega[:, 1:] += np.diff(uy, axis=1)
    omega *= mesh.slipcoef


def compute_kinetic_energy(p, mesh, ux, uy, Ux, Uy, ke, pysq):
    """operators.py:80-96: the 4-point product of innerproduct="classic"
    (86-90) or the WENO inner product of the other methods (92-96)."""
    ke[:] = 0.
    if p.innerproduct == "classic":
        ke[:, :-1] = +ux[:, 1:] * Ux[:, 1:] + ux[:, :-1] * Ux[:, :-1]
        ke[:-1, :] += uy[1:, :] * Uy[1:, :] + uy[:-1, :] * Uy[:-1, :]
        ke *= mesh.msk * 0.25
        return
    innerproduct(ke, Ux, ux, mesh.okx, mesh.xshift, p.innerproduct, pysq)
    innerproduct(ke, Uy, uy, mesh.oky, mesh.yshift, p.innerproduct, pysq)
    ke *= mesh.msk * 0.5


def div_vector(mesh, Ux, Uy, delta):
    """div (operators.py:104-107) of a vector field; delta's last column
    keeps its previous value, as in the reference."""
    delta[:, :-1] = -np.diff(Ux, axis=1)
    delta[:-1, :] -= np.diff(Uy, axis=0)
    delta *= mesh.msk


def pressure_projection(mesh, Ux, Uy, delta, p, ux, uy):
    """operators.py:114-119."""
    sharp(mesh, ux, uy, Ux, Uy)
    div_vector(mesh, Ux, Uy, delta)
    mesh.poisson_centers.solve(-delta * mesh.area, p)
    addgrad(mesh, p, ux, uy)
    mesh.fill(ux)
    mesh.fill(uy)


def compute_pressure(p, mesh, h, out):
    """operators.py:110-111."""
    out[:] = (p.g / mesh.area) * (h + mesh.hb)


def centerstovertices(mesh, c, v):
    """operators.py:126-133 (addto=False)."""
    v[1:, 1:] = 0.25 * (c[:-1, :-1] + c[1:, :-1] + c[:-1, 1:] + c[1:, 1:])
    v *= mesh.mskv


def centerstovertices_add(mesh, c, v):
    """operators.py:126-129, 133 (addto=True)."""
    v[1:, 1:] += 0.25 * (c[:-1, :-1] + c[1:, :-1] + c[:-1, 1:] + c[1:, 1:])
    v *= mesh.mskv


def verticestocenters(mesh, vh, h):
    """operators.py:136-141. A cell with no wet vertex gets (1/0) * 0 = nan,
    as in the reference."""
    m = mesh.mskv
    coef = m[:-1, :-1] + m[1:, :-1] + m[:-1, 1:] + m[1:, 1:]
    with np.errstate(divide="ignore", invalid="ignore"):
        h[:-1, :-1] = (1 / coef) * (vh[:-1, :-1] + vh[1:, :-1] + vh[:-1, 1:]
                                    + vh[1:, 1:])
        h *= mesh.msk


def qg_projection(mesh, ux, uy, h, pv, psi, anomaly=False):
    """operators.py:176-183 with add_stretching (194-201) and
    thickness_from_psi (204-211): project (u, h) on the QG manifold through
    the Helmholtz solve of the PV."""
    p = mesh.param
    f0, H, g = p.f0, p.H, p.g
    compute_vorticity(mesh, ux, uy, pv)
    if anomaly:
        centerstovertices_add(mesh, h * (-f0 / H), pv)
    else:
        h0 = H * mesh.area - mesh.hb
        centerstovertices_add(mesh, (h - h0) * (-f0 / H), pv)
    mesh.qg_helmholtz.solve(pv, psi)
    verticestocenters(mesh, psi * (f0 * mesh.area / g), h)
    if not anomaly:
        h += (H * mesh.area) - mesh.hb
    with np.errstate(invalid="ignore"):
        h *= mesh.msk
    perpgrad(mesh, psi, ux, uy)


def perpgrad(mesh, psi, Ux, Uy, contravariant=False):
    """operators.py:144-149."""
    Ux[:-1, :] = -np.diff(psi, axis=0) * mesh.mskx[:-1, :]
    Uy[:, :-1] = np.diff(psi, axis=1) * mesh.msky[:, :-1]
    if contravariant:
        Ux[:] *= (1 / mesh.dy ** 2)
        Uy[:] *= (1 / mesh.dx ** 2)


# ------------------------------------------------------------- model -----

STATE_VARS = {
    "euler": ("u", "U", "omega", "ke", "p", "div", "flx"),
    "boussinesq": ("b", "u", "U", "omega", "ke", "p", "div", "flx"),
    # states.py:7-17 (the models on the hot path); vector fields get .x/.y
    "eulerpsi": ("omega", "U", "psi", "vomega", "flx"),
    "rsw": ("u", "h", "U", "omega", "ke", "p", "flx", "pv"),
    "qg": ("pv", "U", "h", "flx", "work", "psi"),
    "qgrsw": ("u", "h", "U", "omega", "ke", "p", "flx", "pv", "psi"),
}
PROGNOSTIC = {"eulerpsi": ("omega",), "rsw": ("u", "h"), "qg": ("pv",),
              "euler": ("u",), "boussinesq": ("b", "u"), "qgrsw": ("u", "h")}
VECTORS = ("u", "U", "flx")


class _View:
    """Attribute access to a state dict the way the reference's namedtuples
    give it (s.b, ds.u.y, ...), for forcing functions; arrays are the dict's
    own, so in-place updates reach it."""

    def __init__(self, d):
        self._d = d

    def __getattr__(self, name):
        d = self.__dict__["_d"]
        if name in d:
            return d[name]
        if name + ".x" in d:
            return _Vec(d[name + ".x"], d[name + ".y"])
        raise AttributeError(name)


class _Vec:
    def __init__(self, x, y):
        self.x, self.y = x, y


def _alloc(names, shape):
    out = {}
    for n in names:
        if n in VECTORS:
            out[n + ".x"] = np.zeros(shape)
            out[n + ".y"] = np.zeros(shape)
        else:
            out[n] = np.zeros(shape)
    return out


class Model:
    """Model + RKIntegrator(rk3) + the eulerpsi/rsw/qg equation sets
    (model.py:13-87, integrators.py:63-107, equations.py:73-157)."""

    def __init__(self, param, msk=None, pysq=True):
        self.p = param
        self.pysq = pysq
        self.mesh = Mesh(param)
        if msk is not None:
            self.mesh.msk[:] = msk
            self.mesh.finalize()
        shape = self.mesh.shape
        tr = getattr(param, "tracer", None)
        self.tracer = None if tr in (None, "None") else tr
        self.s = _alloc(STATE_VARS[param.model], shape)
        self.prog = [k for k in self.s
                     if k.split(".")[0] in PROGNOSTIC[param.model]]
        if self.tracer:
            # states.py:31-34: the tracer is the last prognostic variable
            self.s[self.tracer] = np.zeros(shape)
            self.prog.append(self.tracer)
        self.scratch = [{k: np.zeros(shape) for k in self.prog}
                        for _ in range(3)]
        self.t = 0.0
        self.ite = 0
        self._c = 0.0
        self.dt = param.dt if param.dt > 0 else 0.01
        self.forcings = []

    @property
    def param(self):
        return self.p

    def add_forcing(self, forcing):
        """Model.add_forcing (model.py:121-123): forcing(param, mesh, s, ds)
        runs after the right-hand side (addforcingterm, equations.py:229-238);
        several are applied in the order they were added."""
        self.forcings.append(forcing)

    # -- equations ------------------------------------------------------
    def rhs(self, s, ds):
        p, m, sq = self.p, self.mesh, self.pysq
        if p.model == "eulerpsi":
            divflux(p, m, s["flx.x"], s["flx.y"], s["omega"], s["U.x"],
                    s["U.y"], ds["omega"], sq)
            m.fill(ds["omega"])
        elif p.model == "qg":
            divflux(p, m, s["flx.x"], s["flx.y"], s["pv"], s["U.x"],
                    s["U.y"], ds["pv"], sq)
            m.fill(ds["pv"])
        elif p.model == "rsw":
            addvortexforce(p, m, s["U.x"], s["U.y"], s["omega"], ds["u.x"],
                           ds["u.y"], sq)
            addcoriolis(p, m, s["U.x"], s["U.y"], ds["u.x"], ds["u.y"])
            addgrad(m, s["ke"], ds["u.x"], ds["u.y"])
            addgrad(m, s["p"], ds["u.x"], ds["u.y"])
            divflux(p, m, s["flx.x"], s["flx.y"], s["h"], s["U.x"], s["U.y"],
                    ds["h"], sq)
            for k in ("u.x", "u.y", "h"):
                m.fill(ds[k])
        elif p.model == "euler":
            # equations.py:11-15
            addvortexforce(p, m, s["U.x"], s["U.y"], s["omega"], ds["u.x"],
                           ds["u.y"], sq)
            addgrad(m, s["ke"], ds["u.x"], ds["u.y"])
            for k in ("u.x", "u.y"):
                m.fill(ds[k])
        elif p.model == "boussinesq":
            # equations.py:29-35
            addvortexforce(p, m, s["U.x"], s["U.y"], s["omega"], ds["u.x"],
                           ds["u.y"], sq)
            addgrad(m, s["ke"], ds["u.x"], ds["u.y"])
            addbuoyancy(m, s["b"], ds["u.y"])
            divflux(p, m, s["flx.x"], s["flx.y"], s["b"], s["U.x"], s["U.y"],
                    ds["b"], sq)
            for k in ("u.x", "u.y", "b"):
                m.fill(ds[k])

        elif p.model == "qgrsw":
            # equations.py:106-125: the RSW tendency without the gradient
            # forces, projected on the QG manifold (anomaly form)
            addvortexforce(p, m, s["U.x"], s["U.y"], s["omega"], ds["u.x"],
                           ds["u.y"], sq)
            addcoriolis(p, m, s["U.x"], s["U.y"], ds["u.x"], ds["u.y"])
            divflux(p, m, s["flx.x"], s["flx.y"], s["h"], s["U.x"], s["U.y"],
                    ds["h"], sq)
            qg_projection(m, ds["u.x"], ds["u.y"], ds["h"], s["pv"], s["psi"],
                          anomaly=True)
            for k in ("u.x", "u.y", "h"):
                m.fill(ds[k])
        if self.tracer:
            # addtracerequation (equations.py:217-226): no halo fill
            divflux(p, m, s["flx.x"], s["flx.y"], s[self.tracer], s["U.x"],
                    s["U.y"], ds[self.tracer], sq)
        for f in self.forcings:
            f(p, m, _View(s), _View(ds))

    def diag(self, s=None):
        s = self.s if s is None else s
        p, m, sq = self.p, self.mesh, self.pysq
        if p.model == "eulerpsi":
            centerstovertices(m, s["omega"], s["vomega"])
            m.poisson_vertices.solve(s["vomega"], s["psi"])
            perpgrad(m, s["psi"], s["U.x"], s["U.y"], contravariant=True)
            m.fill(s["U.x"])
            m.fill(s["U.y"])
        elif p.model == "qg":
            pvback = m.hb * m.qgcoef
            centerstovertices(m, s["pv"] - pvback, s["work"])
            if p.beta != 0:
                s["work"] -= m.f
            m.qg_helmholtz.solve(s["work"], s["psi"])
            perpgrad(m, s["psi"], s["U.x"], s["U.y"], contravariant=True)
        elif p.model in ("euler", "boussinesq"):
            # equations.py:17-22; the boussinesq diag (37-43) is the same:
            # its fill(s.u) passes no mesh and fills nothing
            pressure_projection(m, s["U.x"], s["U.y"], s["div"], s["p"],
                                s["u.x"], s["u.y"])
            sharp(m, s["u.x"], s["u.y"], s["U.x"], s["U.y"])
            compute_vorticity(m, s["u.x"], s["u.y"], s["omega"])
            compute_kinetic_energy(p, m, s["u.x"], s["u.y"], s["U.x"],
                                   s["U.y"], s["ke"], sq)
            m.fill(s["omega"])
            m.fill(s["ke"])
        elif p.model == "qgrsw":
            # equations.py:127-133
            sharp(m, s["u.x"], s["u.y"], s["U.x"], s["U.y"])
            compute_vorticity(m, s["u.x"], s["u.y"], s["omega"])
            m.fill(s["omega"])
        elif p.model == "rsw":
            sharp(m, s["u.x"], s["u.y"], s["U.x"], s["U.y"])
            compute_vorticity(m, s["u.x"], s["u.y"], s["omega"])
            compute_kinetic_energy(p, m, s["u.x"], s["u.y"], s["U.x"],
                                   s["U.y"], s["ke"], sq)
            compute_pressure(p, m, s["h"], s["p"])
            m.fill(s["omega"])
            m.fill(s["ke"])

    # -- integrator -----------------------------------------------------
    def _addto(self, coefs, dss):
        """addto_list, integrators.py:154-174: y += sum(c*x)."""
        for k in self.prog:
            self.s[k][:] += sum((c * d[k] for c, d in zip(coefs, dss)))

    def rk3(self, dt):
        """integrators.py:92-107."""
        ds1, ds2, ds3 = self.scratch
        self.rhs(self.s, ds1)
        self._addto([dt], [ds1])
        self.diag()
        self.rhs(self.s, ds2)
        self._addto([-3 * dt / 4, dt / 4], [ds1, ds2])
        self.diag()
        self.rhs(self.s, ds3)
        self._addto([-dt / 12, -dt / 12, 2 * dt / 3], [ds1, ds2, ds3])
        self.diag()

    def ef(self, dt):
        """integrators.py:116-123."""
        (ds1,) = self.scratch[:1]
        self.rhs(self.s, ds1)
        self._addto([dt], [ds1])
        self.diag()

    def enrk3(self, dt):
        """integrators.py:140-155."""
        ds1, ds2, ds3 = self.scratch
        self.rhs(self.s, ds1)
        self._addto([dt / 3], [ds1])
        self.diag()
        self.rhs(self.s, ds2)
        self._addto([-dt / 3 - 5 * dt / 48, 15 * dt / 16], [ds1, ds2])
        self.diag()
        self.rhs(self.s, ds3)
        self._addto([5 * dt / 48 + dt / 10, -7 * dt / 16, 2 * dt / 5], [ds1, ds2, ds3])
        self.diag()

    def lfra(self, dt):
        """integrators.py:39-55 (LFRA) with rightpermute (134-137): Euler
        forward at ite == 0 (sb = sa = s), then sa += 2 dt ds;
        s += gamma sa + gamma sb - 2 gamma s; (sb, s, sa) <- (s, sa, s)."""
        sb, sa, ds = self.scratch
        gam = getattr(self.p, "RAgamma", 0.1)
        self.rhs(self.s, ds)
        if self.ite == 0:
            for k in self.prog:
                sb[k][:] = self.s[k]
                sa[k][:] = self.s[k]
            self._addto([dt], [ds])
        else:
            for k in self.prog:
                sa[k][:] += sum((c * d[k] for c, d in zip([2 * dt], [ds])))
            self._addto([gam, gam, -2 * gam], [sa, sb, self.s])
            for k in self.prog:
                sb[k][:] = self.s[k]
                self.s[k][:] = sa[k]
                sa[k][:] = sb[k]
        self.diag()

    def pushforward(self):
        """timeline.py:20-35 (Kahan-summed time)."""
        y = self.dt - self._c
        t = self.t + y
        self._c = (t - self.t) - y
        self.t = t
        self.ite += 1

    def set_dt(self):
        """model.py:71-87."""
        p = self.p
        if p.dt > 0:
            self.dt = p.dt
            return
        if p.model == "rsw":
            c = (p.g * p.H) ** 0.5
            maxU = c / self.mesh.dx + c / self.mesh.dy
        else:
            maxU = (np.max(np.abs(self.s["U.x"])) +
                    np.max(np.abs(self.s["U.y"])) + 1e-99)
        self.dt = min(p.cfl / maxU, p.dtmax)

    def step(self, n=1):
        integ = {"rk3": self.rk3, "ef": self.ef, "enrk3": self.enrk3,
                 "LFRA": self.lfra}[getattr(self.p, "integrator", "rk3")]
        for _ in range(n):
            integ(self.dt)
            self.pushforward()

    def run_steps(self, n):
        """n iterations of the Model.run loop body: set_dt then step(1)."""
        dts = []
        for _ in range(n):
            self.set_dt()
            dts.append(self.dt)
            self.step(1)
        return dts


def bulk(m):
    """Bulk.__call__ (diagnostics.py:44-57) on an oracle model: (t, ke, ens,
    vort, angular) with domavg = sum over the whole array / sum(msk) and the
    y-face x / x-face y coordinates of meshes.py:57-68."""
    mesh, s = m.mesh, m.s
    h = m.p.halowidth
    S = np.sum(mesh.msk, axis=None)

    def domavg(x):
        return np.sum(x, axis=None) / S

    ix = np.arange(mesh.nx + 2 * h) - h
    iy = np.arange(mesh.ny + 2 * h) - h
    xv, _ = np.meshgrid((ix + 0.5) * mesh.dx, iy * mesh.dy)
    _, yu = np.meshgrid(ix * mesh.dx, (iy + 0.5) * mesh.dy)
    area = mesh.area
    return (m.t, domavg(s["ke"]), 0.5 * domavg(s["omega"] ** 2) / area ** 2,
            domavg(s["omega"]) / area,
            domavg(s["U.y"] * xv) * mesh.dx - domavg(s["U.x"] * yu) * mesh.dy)


def num_threads():
    return int(lib().oracle_num_threads())


def rel_l2(a, b, mask=None):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if mask is not None:
        a = a[mask]
        b = b[mask]
    nb = math.sqrt(float(np.sum(b * b)))
    d = math.sqrt(float(np.sum((a - b) ** 2)))
    return d / nb if nb > 0 else d
