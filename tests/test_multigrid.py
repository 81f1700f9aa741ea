"""The multigrid preconditioner itself, through the Poisson solve.

A preconditioned CG converges to the same solution with a poor or even a
wrong symmetric preconditioner, only in more iterations, so the parity tests
of the solution cannot see a broken V-cycle. These tests bound the iteration
count of solves from a zero initial guess to the 1e-12 relative residual on
grids with islands, x-periodic channels and the Helmholtz operator, for both
forms and every multigrid schedule (1 or 2 sweeps per leg, 32- or 64-row
tiles), and check the solution against the plain sparse operator; the FP32
form runs the pipelined level kernels (mg_pipe.cuh), the FP64 form the
one-tile-per-block ones (mg_reg.cuh).
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from fluids2d_gb300 import workloads as wl  # noqa: E402
from fluids2d_gb300._lib import lib  # noqa: E402
from test_gpu_parity import _model  # noqa: E402

# a V-cycle with red-black Gauss-Seidel reduces the residual by about 10x per
# CG iteration on these grids; 12 orders of magnitude take 8-14 iterations
MAX_ITERS = {"fp64": 20, "fp32": 40}


def _case(kind, n):
    if kind == "islands":
        c = wl.eulerpsi_case(n=n, seed=5, nislands=4)
        return c, "eulerpsi", dict()
    if kind == "periodic":
        c = wl.rsw_case(n=n, seed=6, nislands=3, xperiodic=True)
        return c, "qg", dict(xperiodic=True, f0=0.0)
    c = wl.qg_case(n=n, seed=7, nislands=6)
    return c, "qg", dict(f0=c["f0"])


@pytest.mark.parametrize("schedule", [(32, 2), (64, 2), (32, 1), (64, 1)])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("kind,n", [("islands", 256), ("islands", 512),
                                    ("periodic", 384), ("helmholtz", 512)])
def test_poisson_iterations_from_zero(kind, n, precision, schedule):
    case, model, kw = _case(kind, n)
    m = _model(model, n, n, case["msk"], precision=precision, **kw)
    m.set_schedule(*schedule)
    solver = m.mesh.qg_helmholtz if model == "qg" else m.mesh.poisson_vertices
    rng = np.random.default_rng(11)
    b = rng.standard_normal(m.mesh.shape) * (m.mesh.G_vertices >= 0)
    x = np.zeros(m.mesh.shape)
    solver.solve(b, x)
    it = solver.last_iters
    print(f"{kind} {n}^2 {precision} {schedule}: {it} iterations, "
          f"relres {solver.last_relres:.1e}")
    assert it <= MAX_ITERS[precision], it
    # the FP32 form runs the pipelined level kernels on these layouts (the
    # periodic channel's edge tiles through their element-wise path)
    pipe = ctypes.c_int(-1)
    assert lib().f2d_solver_pipelined(m._h, ctypes.byref(pipe)) == 0
    assert pipe.value == (1 if precision == "fp32" else 0)
    # the true residual with the sparse operator
    om = O.Mesh(O.Param(model=model, nx=n, ny=n, xperiodic=kw.get("xperiodic", False),
                        f0=kw.get("f0", 0.0), g=1.0, H=1.0))
    om.msk[:] = case["msk"]
    om.finalize()
    md = om.maindiag if model == "qg" else 0.0
    A, G = O.laplacian(om, md)[:2]
    sel = G >= 0
    r = b[sel] - A @ x[sel]
    assert np.linalg.norm(r) <= 1e-10 * np.linalg.norm(b[sel])
