"""Seeded synthetic workloads: masks and initial conditions.

These are the recipes the benchmarks and the parity tests share. They follow
the forms of the reference's experiment scripts, without copying them:

* Gaussian vortices on cell centres, multiplied by ``msk * area``
  (form of ``src/experiments/vortex.py:5, 23-26``);
* circular islands carved into ``msk`` followed by ``mesh.finalize()``
  (form of ``src/experiments/vortex.py:45-51``);
* a Gaussian thickness bump for the shallow-water model, ``h * msk * area``
  (form of ``src/experiments/inpreparation/rsw_with_topo.py:12-37``);
* a beta-plane Coriolis term ``beta*(y - Ly/2)*area`` added to the potential
  vorticity (form of ``src/experiments/inpreparation/gyre.py:109-120``).

Every function takes an explicit ``seed`` and draws from
``numpy.random.default_rng(seed)``, so the same call gives the same arrays on
any machine.
"""
from __future__ import annotations

import numpy as np


def grid_coords(nx, ny, Lx, Ly, halowidth=3, which="c"):
    """Coordinates of the (ny+2h, nx+2h) array points.

    ``which`` is "c" (cell centres), "v" (vertices), "x" (x-faces) or "y"
    (y-faces), as in ``meshes.py:57-68`` of the reference: index
    ``arange(n+2h) - h``, shifted by one half where the location is centred.
    """
    dx, dy = Lx / nx, Ly / ny
    ix = np.arange(nx + 2 * halowidth) - halowidth
    iy = np.arange(ny + 2 * halowidth) - halowidth
    sx = 0.5 if which in ("c", "y") else 0.0
    sy = 0.5 if which in ("c", "x") else 0.0
    return np.meshgrid((ix + sx) * dx, (iy + sy) * dy)


def carve_islands(msk, x, y, nislands, rmin, rmax, seed, Lx=1.0, Ly=1.0,
                  margin=None):
    """Zero ``msk`` inside ``nislands`` random discs (in place).

    Centres are uniform in ``[margin, L-margin]`` (default margin = rmax),
    radii uniform in ``[rmin, rmax]`` (in units of length).
    Returns the list of (xc, yc, r).
    """
    rng = np.random.default_rng(seed)
    if margin is None:
        margin = rmax
    out = []
    for _ in range(nislands):
        xc = rng.uniform(margin, Lx - margin)
        yc = rng.uniform(margin, Ly - margin)
        r = rng.uniform(rmin, rmax)
        msk[(x - xc) ** 2 + (y - yc) ** 2 < r ** 2] = 0
        out.append((xc, yc, r))
    return out


def gaussian_vortices(x, y, nvortices, radius, seed, Lx=1.0, Ly=1.0):
    """Sum of ``nvortices`` Gaussians of amplitude +-1 and given radius.

    Centres are uniform in the interior ``[radius, L-radius]``; the sign of
    each vortex is drawn from the same generator.
    """
    rng = np.random.default_rng(seed)
    w = np.zeros_like(x)
    for _ in range(nvortices):
        xc = rng.uniform(radius, Lx - radius)
        yc = rng.uniform(radius, Ly - radius)
        sgn = 1.0 if rng.uniform() < 0.5 else -1.0
        w += sgn * np.exp(-((x - xc) ** 2 + (y - yc) ** 2) / (2 * radius ** 2))
    return w


def band_limited_field(nx, ny, kmin, kmax, seed, halowidth=3):
    """Gaussian random field on the nx*ny interior with |k| in [kmin, kmax].

    Built in Fourier space with random phases and a flat spectrum inside the
    annulus, then scaled to unit variance. The returned array has the full
    (ny+2h, nx+2h) shape with zeros in the halo.
    """
    rng = np.random.default_rng(seed)
    kx = np.fft.fftfreq(nx, 1.0 / nx)
    ky = np.fft.fftfreq(ny, 1.0 / ny)
    KX, KY = np.meshgrid(kx, ky)
    K = np.hypot(KX, KY)
    amp = ((K >= kmin) & (K <= kmax)).astype(float)
    phase = rng.uniform(0, 2 * np.pi, size=K.shape)
    spec = amp * np.exp(1j * phase)
    f = np.real(np.fft.ifft2(spec))
    f -= f.mean()
    f /= f.std()
    out = np.zeros((ny + 2 * halowidth, nx + 2 * halowidth))
    out[halowidth:-halowidth, halowidth:-halowidth] = f
    return out


# ---------------------------------------------------------------------------
# Whole-config recipes. Each returns a dict of plain numpy arrays and scalars
# so the same inputs feed the GPU model, the oracle and the golden generator.
# ---------------------------------------------------------------------------

def default_mask(nx, ny, halowidth=3, xperiodic=False):
    """Default mask: interior = 1, halo = 1 only in a periodic direction
    (``meshes.py:70-75``)."""
    msk = np.zeros((ny + 2 * halowidth, nx + 2 * halowidth), dtype=np.int8)
    xs = slice(None) if xperiodic else slice(halowidth, -halowidth)
    msk[halowidth:-halowidth, xs] = 1
    return msk


def eulerpsi_case(n=256, seed=0, nislands=0, nvortices=8, radius=0.05,
                  ny=None, Lx=1.0, Ly=1.0):
    """Euler vorticity/streamfunction on a closed basin.

    omega = sum of Gaussian vortices * msk * area on cell centres.
    """
    nx = n
    ny = n if ny is None else ny
    x, y = grid_coords(nx, ny, Lx, Ly, which="c")
    msk = default_mask(nx, ny)
    if nislands:
        carve_islands(msk, x, y, nislands, 0.03 * Lx, 0.08 * Lx, seed + 1000,
                      Lx, Ly, margin=0.1 * Lx)
    area = (Lx / nx) * (Ly / ny)
    omega = gaussian_vortices(x, y, nvortices, radius * Lx, seed, Lx, Ly)
    omega = omega * msk * area
    return dict(model="eulerpsi", nx=nx, ny=ny, Lx=Lx, Ly=Ly, msk=msk,
                fields={"omega": omega})


def rsw_case(n=512, seed=0, nislands=3, ny=None, Lx=1.0, Ly=1.0,
             f0=1.0, g=1.0, H=1.0, xperiodic=True):
    """Rotating shallow water in an x-periodic channel (or a closed basin)
    with islands.

    h = (H + 0.1*Gaussian bump of radius 0.1 L + N(0, 1e-3)) * msk * area,
    u = 0.
    """
    nx = n
    ny = n if ny is None else ny
    x, y = grid_coords(nx, ny, Lx, Ly, which="c")
    msk = default_mask(nx, ny, xperiodic=xperiodic)
    carve_islands(msk, x, y, nislands, 0.03 * Lx, 0.08 * Lx, seed + 1000,
                  Lx, Ly, margin=0.1 * Lx)
    rng = np.random.default_rng(seed)
    area = (Lx / nx) * (Ly / ny)
    r0 = 0.1 * Lx
    bump = np.exp(-((x - 0.5 * Lx) ** 2 + (y - 0.5 * Ly) ** 2) / (2 * r0 ** 2))
    h = (H + 0.1 * bump + rng.normal(0.0, 1e-3, size=x.shape)) * msk * area
    if xperiodic:
        # periodic halo columns hold copies of the interior (the halo fill)
        hw = 3
        h[:, :hw] = h[:, -2 * hw:-hw]
        h[:, -hw:] = h[:, hw:2 * hw]
    return dict(model="rsw", nx=nx, ny=ny, Lx=Lx, Ly=Ly, msk=msk,
                xperiodic=xperiodic, f0=f0, g=g, H=H, fields={"h": h})


def add_tracer(case, name="q", seed=0, nblobs=3):
    """A passive tracer field `name` (param.tracer) on top of a case: a sum
    of Gaussian blobs plus a smooth gradient, masked by msk, with the
    x-periodic halo fill where the case is x-periodic."""
    nx, ny, Lx, Ly = case["nx"], case["ny"], case["Lx"], case["Ly"]
    x, y = grid_coords(nx, ny, Lx, Ly, which="c")
    rng = np.random.default_rng(seed + 77)
    q = 0.5 * (x / Lx)
    for _ in range(nblobs):
        x0, y0 = rng.uniform(0.2, 0.8) * Lx, rng.uniform(0.2, 0.8) * Ly
        r0 = rng.uniform(0.05, 0.12) * Lx
        q = q + np.exp(-((x - x0) ** 2 + (y - y0) ** 2) / r0 ** 2)
    q = q * case["msk"]
    if case.get("xperiodic"):
        hw = 3
        q[:, :hw] = q[:, -2 * hw:-hw]
        q[:, -hw:] = q[:, hw:2 * hw]
    out = dict(case)
    out["fields"] = dict(case["fields"])
    out["fields"][name] = q
    out["tracer"] = name
    return out


def qg_case(n=4096, seed=0, nislands=20, ny=None, Lx=1.0, Ly=1.0,
            Rd=0.02, beta=1.0, g=1.0, H=1.0, kmin=4, kmax=32):
    """Quasi-geostrophic PV on a closed basin with islands and a beta-plane.

    f0 = sqrt(g H)/(Rd L). pv = area*(q' + beta*(y - Ly/2)) * msk with q' a
    unit-variance band-limited field, and the vertex Coriolis term
    f = beta*(y_v - Ly/2)*area.
    """
    nx = n
    ny = n if ny is None else ny
    x, y = grid_coords(nx, ny, Lx, Ly, which="c")
    msk = default_mask(nx, ny)
    carve_islands(msk, x, y, nislands, 0.01 * Lx, 0.04 * Lx, seed + 1000,
                  Lx, Ly, margin=0.05 * Lx)
    area = (Lx / nx) * (Ly / ny)
    f0 = np.sqrt(g * H) / (Rd * Lx)
    q = band_limited_field(nx, ny, kmin, kmax, seed)
    pv = (q + beta * (y - Ly / 2)) * area * msk
    xv, yv = grid_coords(nx, ny, Lx, Ly, which="v")
    fv = beta * (yv - Ly / 2) * area
    return dict(model="qg", nx=nx, ny=ny, Lx=Lx, Ly=Ly, msk=msk, f0=f0,
                beta=beta, g=g, H=H, fields={"pv": pv}, f=fv)


def euler_case(n=128, seed=0, nislands=2, ny=None, Lx=1.0, Ly=1.0, xperiodic=False,
               nvortices=6, radius=0.08, noise=0.05):
    """Euler (momentum-pressure form) with an initial velocity that is not
    divergence-free: the covariant velocity of a streamfunction made of
    Gaussian vortices (form of vortex.py's initial condition) plus a random
    divergent part of relative size `noise`, masked by mskx/msky, so that the
    first diagnostic's pressure projection has work to do."""
    nx = n
    ny = n if ny is None else ny
    x, y = grid_coords(nx, ny, Lx, Ly, which="c")
    msk = default_mask(nx, ny, xperiodic=xperiodic)
    if nislands:
        carve_islands(msk, x, y, nislands, 0.03 * Lx, 0.08 * Lx, seed + 1000,
                      Lx, Ly, margin=0.1 * Lx)
    xv, yv = grid_coords(nx, ny, Lx, Ly, which="v")
    psi = gaussian_vortices(xv, yv, nvortices, radius * Lx, seed, Lx, Ly)
    psi *= (Lx / nx) * (Ly / ny) * 0.5
    mx = np.zeros_like(msk)
    mx[:, 1:] = msk[:, 1:] * msk[:, :-1]
    my = np.zeros_like(msk)
    my[1:, :] = msk[1:, :] * msk[:-1, :]
    ux = np.zeros(msk.shape)
    uy = np.zeros(msk.shape)
    ux[:-1, :] = -(psi[1:, :] - psi[:-1, :])
    uy[:, :-1] = psi[:, 1:] - psi[:, :-1]
    rng = np.random.default_rng(seed + 7)
    scale = noise * max(np.abs(ux).max(), np.abs(uy).max(), 1e-300)
    ux = (ux + scale * rng.standard_normal(msk.shape)) * mx
    uy = (uy + scale * rng.standard_normal(msk.shape)) * my
    if xperiodic:
        hw = 3
        for a in (ux, uy):
            a[:, :hw] = a[:, -2 * hw:-hw]
            a[:, -hw:] = a[:, hw:2 * hw]
    return dict(model="euler", nx=nx, ny=ny, Lx=Lx, Ly=Ly, msk=msk,
                xperiodic=xperiodic, fields={"u.x": ux, "u.y": uy})


def boussinesq_case(n=128, seed=0, nislands=2, ny=None, Lx=1.0, Ly=1.0,
                    xperiodic=False, nbubbles=2, strat=0.5, **kw):
    """Boussinesq (momentum-pressure form with buoyancy b): the velocity of
    euler_case plus a buoyancy field of a stable linear stratification and
    Gaussian bubbles, masked by msk. The amplitude is set so that the
    buoyancy force changes u by about a tenth of its size per CFL step."""
    c = euler_case(n=n, seed=seed, nislands=nislands, ny=ny, Lx=Lx, Ly=Ly,
                   xperiodic=xperiodic, **kw)
    nx, ny = c["nx"], c["ny"]
    x, y = grid_coords(nx, ny, Lx, Ly, which="c")
    rng = np.random.default_rng(seed + 31)
    dx, dy = Lx / nx, Ly / ny
    umax = max(np.abs(c["fields"]["u.x"]).max(), np.abs(c["fields"]["u.y"]).max(),
               1e-300)
    amp = 0.1 * umax ** 2 / (dy * dx ** 2)
    b = strat * amp * (y / Ly - 0.5)
    for _ in range(nbubbles):
        x0, y0 = rng.uniform(0.2, 0.8) * Lx, rng.uniform(0.2, 0.5) * Ly
        r0 = rng.uniform(0.06, 0.12) * Lx
        b = b + amp * rng.choice([-1.0, 1.0]) * np.exp(-((x - x0) ** 2 + (y - y0) ** 2)
                                                      / r0 ** 2)
    b = b * c["msk"]
    if xperiodic:
        hw = 3
        b[:, :hw] = b[:, -2 * hw:-hw]
        b[:, -hw:] = b[:, hw:2 * hw]
    c["model"] = "boussinesq"
    c["fields"]["b"] = b
    return c


def ensemble_case(count=256, seed=0, sizes=(64, 128, 192, 256, 384, 512),
                  max_islands=4, nvortices=8, radius=0.05):
    """Batched ensemble of closed-basin eulerpsi members: grid sizes drawn
    uniformly from `sizes`, 0..max_islands islands each, Gaussian-vortex
    initial vorticity as in eulerpsi_case."""
    rng = np.random.default_rng(seed)
    members = []
    for b in range(count):
        n = int(rng.choice(sizes))
        k = int(rng.integers(0, max_islands + 1))
        members.append(eulerpsi_case(n=n, seed=seed * 100003 + b, nislands=k,
                                     nvortices=nvortices, radius=radius))
    return members
