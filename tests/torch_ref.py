"""Plain-torch FP64 restatement of the eulerpsi time step, for checking the
adjoint kernels (test infrastructure, never part of the product path).

Forward map, written with differentiable torch ops so that autograd gives
the reference gradient:

* centerstovertices (operators.py:126-133), the vertex Poisson solve with
  Dirichlet walls (elliptic.py:71-87, the same matrix as the oracle's,
  solved densely), perpgrad with contravariant scaling (operators.py:144-149);
* the flux-form tendency -div(phi(U, omega) U) * msk with the face order
  levels of the mesh (compflux_on_interval, weno.py:346-364; upwind side by
  the sign of U; weno5z / weno3z / first-order upwind for the weno method,
  weno.py:75-100, 167-197, 303-343) and div (operators.py:104-107);
* SSP-RK3 in increment form (integrators.py:92-107) with a fixed dt.

Masks, order arrays and the Poisson matrix come from the oracle's Mesh
(oracle/oracle.py), so the torch forward is pinned to the oracle forward by
the tests. Closed (non-periodic) basins only.
"""
from __future__ import annotations

import numpy as np
import torch
import torch.nn.functional as F


def _level(o):
    """order value -> level 3 (f5), 2 (f3), 1 (f1), 0 (no flux)."""
    return np.where(o > 4, 3, np.where(o > 2, 2, np.where(o > 0, 1, 0)))


def weno5z(a, b, c, d, e):
    eps = 1e-16
    qi1 = (a / 3 - 7 * b / 6) + 11 * c / 6
    qi2 = (-b / 6 + 5 * c / 6) + d / 3
    qi3 = (c / 3 + 5 * d / 6) - e / 6
    k1, k2 = 13. / 12., 0.25
    b1 = k1 * ((a - 2 * b) + c) ** 2 + k2 * ((a - 4 * b) + 3 * c) ** 2
    b2 = k1 * ((b - 2 * c) + d) ** 2 + k2 * (b - d) ** 2
    b3 = k1 * ((c - 2 * d) + e) ** 2 + k2 * ((3 * c - 4 * d) + e) ** 2
    tau = torch.abs(b1 - b3)
    w1 = 0.1 * (1 + tau / (b1 + eps))
    w2 = 0.6 * (1 + tau / (b2 + eps))
    w3 = 0.3 * (1 + tau / (b3 + eps))
    return ((w1 * qi1 + w2 * qi2) + w3 * qi3) / ((w1 + w2) + w3)


def weno3z(a, b, c):
    eps = 1e-14
    qi1 = -0.5 * a + 1.5 * b
    qi2 = 0.5 * (b + c)
    b1 = (b - a) ** 2
    b2 = (c - b) ** 2
    tau = torch.abs(b2 - b1)
    w1 = (1. / 3.) * (1 + tau / (b1 + eps))
    w2 = (2. / 3.) * (1 + tau / (b2 + eps))
    return (w1 * qi1 + w2 * qi2) / (w1 + w2)


class TorchEulerpsi:
    """The eulerpsi step on a closed basin in torch FP64 (CPU)."""

    def __init__(self, mesh, method="weno"):
        assert not mesh.param.xperiodic, "closed basins only"
        assert method in ("weno", "upwind")
        self.method = method
        t = lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64))
        self.msk = t(mesh.msk)
        self.mskx = t(mesh.mskx)
        self.msky = t(mesh.msky)
        self.mskv = t(mesh.mskv)
        self.Lx = torch.as_tensor(_level(mesh.ocx))
        self.Ly = torch.as_tensor(_level(mesh.ocy))
        self.rdx2 = 1 / mesh.dx ** 2
        self.rdy2 = 1 / mesh.dy ** 2
        solver = mesh.poisson_vertices
        self.A = torch.as_tensor(solver.A.toarray())
        G = solver.G
        self.sel = torch.as_tensor(np.flatnonzero(G.ravel() > -1))
        self.shape = mesh.shape

    # -- building blocks -------------------------------------------------
    def psi(self, w):
        v = torch.zeros_like(w)
        v = v.clone()
        avg = 0.25 * (((w[:-1, :-1] + w[1:, :-1]) + w[:-1, 1:]) + w[1:, 1:])
        v = F.pad(avg, (1, 0, 1, 0)) * self.mskv
        b = v.reshape(-1)[self.sel]
        x = torch.linalg.solve(self.A, b)
        psi = torch.zeros(w.numel(), dtype=w.dtype).index_put((self.sel,), x)
        return psi.reshape(w.shape)

    def velocity(self, psi):
        ux = -(psi[1:, :] - psi[:-1, :]) * self.mskx[:-1, :] * self.rdy2
        uy = (psi[:, 1:] - psi[:, :-1]) * self.msky[:, :-1] * self.rdx2
        return F.pad(ux, (0, 0, 0, 1)), F.pad(uy, (0, 1, 0, 0))

    def _faces(self, L, U, win):
        q0, q1, q2, q3, q4, q5 = win
        up = U > 0
        sel = lambda a, b: torch.where(up, a, b)
        if self.method == "weno":
            v3 = weno5z(sel(q0, q5), sel(q1, q4), sel(q2, q3), sel(q3, q2), sel(q4, q1))
            v2 = weno3z(sel(q1, q4), sel(q2, q3), sel(q3, q2))
        else:
            a, b, c, d, e = sel(q0, q5), sel(q1, q4), sel(q2, q3), sel(q3, q2), sel(q4, q1)
            v3 = ((((2 * a - 13 * b) + 47 * c) + 27 * d) - 3 * e) / 60
            a, b, c = sel(q1, q4), sel(q2, q3), sel(q3, q2)
            v2 = ((5 * b + 2 * c) - a) / 6
        v1 = sel(q2, q3)
        z = torch.zeros_like(U)
        phi = torch.where(L == 3, v3, torch.where(L == 2, v2, torch.where(L == 1, v1, z)))
        return phi * U

    def tendency(self, w):
        ux, uy = self.velocity(self.psi(w))
        ny, nx = w.shape
        # 6-point windows: x-face (j,i) sees cells i-3..i+2, zero outside
        wp = F.pad(w, (3, 3, 3, 3))
        winx = [wp[3:3 + ny, k:k + nx] for k in range(6)]
        winy = [wp[k:k + ny, 3:3 + nx] for k in range(6)]
        fx = self._faces(self.Lx, ux, winx)
        fy = self._faces(self.Ly, uy, winy)
        dx = F.pad(-(fx[:, 1:] - fx[:, :-1]), (0, 1, 0, 0))
        dy = F.pad(fy[1:, :] - fy[:-1, :], (0, 0, 0, 1))
        return (dx - dy) * self.msk

    def step(self, w, dt):
        d1 = self.tendency(w)
        y = w + dt * d1
        d2 = self.tendency(y)
        y = y + (-3 * dt / 4 * d1 + dt / 4 * d2)
        d3 = self.tendency(y)
        return y + ((-dt / 12 * d1 + -dt / 12 * d2) + 2 * dt / 3 * d3)

    def rollout(self, w, dt, nsteps):
        for _ in range(nsteps):
            w = self.step(w, dt)
        return w
