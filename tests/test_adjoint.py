"""Discrete adjoint of the eulerpsi step.

CPU (no GPU): the plain-torch FP64 restatement (tests/torch_ref.py) is pinned
to the oracle forward, and its autograd gradient to central finite
differences, so it can serve as the reference gradient.

GPU: the adjoint kernels behind fluids2d_gb300.adjoint.rollout against
(1) the torch reference gradient at small size (rel L2 <= 1e-9, FP64),
(2) central finite differences of the GPU FP64 forward along random
directions (<= 1e-5 relative), (3) the FP32 form's gradient against the FP64
form's (stated tolerance 1e-3: the FP32 trajectory differs from the FP64 one
at the 1e-6 level and the gradient is linearised about it).
"""
import numpy as np
import pytest

from oracle import oracle as O
from fluids2d_gb300 import workloads as wl

torch = pytest.importorskip("torch")
torch_ref = pytest.importorskip("torch_ref")


def _case(nx=24, ny=20, nislands=1, seed=3):
    c = wl.eulerpsi_case(n=nx, ny=ny, nislands=nislands, seed=seed, nvortices=4,
                         radius=0.12)
    return c


def _oracle_model(c, dt, method="weno"):
    p = O.Param(model="eulerpsi", nx=c["nx"], ny=c["ny"], dt=dt, compflux=method)
    m = O.Model(p, msk=c["msk"])
    m.s["omega"][:] = c["fields"]["omega"]
    m.diag()
    return m


def _cfl_dt(m, cfl=0.8):
    return cfl / (np.max(np.abs(m.s["U.x"])) + np.max(np.abs(m.s["U.y"])) + 1e-99)


# ------------------------------------------------------------------ CPU ----
@pytest.mark.parametrize("method", ["weno", "upwind"])
def test_torch_reference_matches_oracle(method):
    c = _case()
    m = _oracle_model(c, 0.0, method)
    dt = _cfl_dt(m)
    m.dt = dt
    ref = torch_ref.TorchEulerpsi(m.mesh, method)
    w0 = torch.as_tensor(c["fields"]["omega"].copy())
    wT = ref.rollout(w0, dt, 3).numpy()
    m.step(3)
    assert O.rel_l2(wT, m.s["omega"]) < 1e-12


def test_torch_reference_gradient_vs_fd():
    c = _case(nx=16, ny=12, nislands=0)
    m = _oracle_model(c, 0.0)
    dt = _cfl_dt(m)
    ref = torch_ref.TorchEulerpsi(m.mesh)
    w0 = torch.as_tensor(c["fields"]["omega"].copy()).requires_grad_(True)
    rng = np.random.default_rng(5)
    lam = torch.as_tensor(rng.standard_normal(w0.shape))
    (g,) = torch.autograd.grad((ref.rollout(w0, dt, 3) * lam).sum(), w0)
    fluid = torch.as_tensor(c["msk"] > 0)
    for k in range(3):
        v = torch.as_tensor(rng.standard_normal(w0.shape)) * fluid
        # WENO-Z is only piecewise smooth (|beta1 - beta3| in the weights):
        # a step small enough not to cross a kink, the direct solve exact
        h = 1e-8 * float(w0.detach().abs().max()) / float(v.abs().max())
        with torch.no_grad():
            fp = (ref.rollout(w0 + h * v, dt, 3) * lam).sum()
            fm = (ref.rollout(w0 - h * v, dt, 3) * lam).sum()
        fd = float(fp - fm) / (2 * h)
        an = float((g * v).sum())
        assert abs(fd - an) <= 1e-5 * abs(an), (k, fd, an)


# ------------------------------------------------------------------ GPU ----
def _gpu_model(c, precision="fp64", method="weno", tol=None):
    import fluids2d_gb300 as f2d
    p = f2d.Param()
    p.model = "eulerpsi"
    p.nx, p.ny = c["nx"], c["ny"]
    p.compflux = method
    p.precision = precision
    if tol is not None:
        p.poisson_tol = tol
    m = f2d.Model(p)
    m.mesh.msk[:] = c["msk"]
    m.mesh.finalize()
    return m


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["weno", "upwind"])
def test_adjoint_matches_torch_reference(method):
    _need_gpu()
    from fluids2d_gb300.adjoint import rollout
    c = _case()
    om = _oracle_model(c, 0.0, method)
    dt = _cfl_dt(om)
    ref = torch_ref.TorchEulerpsi(om.mesh, method)
    w0c = torch.as_tensor(c["fields"]["omega"].copy()).requires_grad_(True)
    nsteps, every = 6, 4  # two checkpoint segments, the second one partial
    wTc = ref.rollout(w0c, dt, nsteps)
    rng = np.random.default_rng(11)
    lam = rng.standard_normal(w0c.shape)
    (gc,) = torch.autograd.grad((wTc * torch.as_tensor(lam)).sum(), w0c)

    m = _gpu_model(c, "fp64", method)
    w0 = torch.tensor(c["fields"]["omega"], device="cuda").requires_grad_(True)
    wT = rollout(m, w0, nsteps, dt, every)
    assert O.rel_l2(wT.detach().cpu().numpy(), wTc.detach().numpy()) < 1e-10
    (g,) = torch.autograd.grad((wT * torch.tensor(lam, device="cuda")).sum(), w0)
    err = O.rel_l2(g.cpu().numpy(), gc.numpy())
    assert err < 1e-9, err


def _loss(wT, target, area):
    return (0.5 * (wT ** 2).mean() + ((wT - target) ** 2).mean()) / area ** 2


@pytest.mark.gpu
def test_adjoint_vs_finite_differences():
    _need_gpu()
    from fluids2d_gb300.adjoint import rollout
    c = _case(nx=48, ny=48, nislands=2, seed=7)
    om = _oracle_model(c, 0.0)
    dt = _cfl_dt(om)
    area = (1.0 / c["nx"]) * (1.0 / c["ny"])
    # finite differences of an iterative solve: the solve's tolerance bounds
    # the noise of the difference quotient (tol / step), so solve to 1e-14
    m = _gpu_model(c, "fp64", tol=1e-14)
    rng = np.random.default_rng(2)
    target = torch.tensor(c["fields"]["omega"] * 0.5, device="cuda")
    w0 = torch.tensor(c["fields"]["omega"], device="cuda").requires_grad_(True)
    nsteps, every = 10, 3
    loss = _loss(rollout(m, w0, nsteps, dt, every), target, area)
    (g,) = torch.autograd.grad(loss, w0)
    fluid = torch.tensor(c["msk"] > 0, device="cuda")
    for k in range(4):
        v = torch.tensor(rng.standard_normal(w0.shape), device="cuda") * fluid
        h = 1e-7 * float(w0.detach().abs().max()) / float(v.abs().max())
        with torch.no_grad():
            fp = _loss(rollout(m, w0 + h * v, nsteps, dt, every), target, area)
            fm = _loss(rollout(m, w0 - h * v, nsteps, dt, every), target, area)
        fd = float(fp - fm) / (2 * h)
        an = float((g * v).sum())
        assert abs(fd - an) <= 1e-5 * abs(an), (k, fd, an)


@pytest.mark.gpu
def test_adjoint_fp32_form_vs_fp64():
    _need_gpu()
    from fluids2d_gb300.adjoint import rollout
    c = _case(nx=64, ny=64, nislands=2, seed=9)
    om = _oracle_model(c, 0.0)
    dt = _cfl_dt(om)
    rng = np.random.default_rng(4)
    lam = torch.tensor(rng.standard_normal((c["ny"] + 6, c["nx"] + 6)), device="cuda")
    grads = {}
    for prec in ("fp64", "fp32"):
        m = _gpu_model(c, prec)
        w0 = torch.tensor(c["fields"]["omega"], device="cuda").requires_grad_(True)
        wT = rollout(m, w0, 8, dt, 4)
        (grads[prec],) = torch.autograd.grad((wT * lam).sum(), w0)
    err = O.rel_l2(grads["fp32"].cpu().numpy(), grads["fp64"].cpu().numpy())
    assert err < 1e-3, err


@pytest.mark.gpu
def test_adjoint_refuses_periodic():
    _need_gpu()
    import fluids2d_gb300 as f2d
    from fluids2d_gb300.adjoint import rollout
    p = f2d.Param()
    p.model = "eulerpsi"
    p.nx, p.ny = 32, 24
    p.xperiodic = True
    m = f2d.Model(p)
    w0 = torch.zeros((30, 38), dtype=torch.float64, device="cuda")
    with pytest.raises(f2d.F2DError):
        rollout(m, w0, 2, 1e-3, 1)
