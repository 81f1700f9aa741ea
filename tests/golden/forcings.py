"""Forcing functions with the reference's signature forcing(param, mesh, s, ds)
(model.py:121-123, equations.py:229-238), in the forms of the reference's
experiment scripts: a constant heating/cooling of the buoyancy rows
(forced_convection.py), a constant wind-curl source of potential vorticity
(gyre.py), a time-periodic momentum source (internalwave_maker.py).

The same functions drive the reference (tests/golden/make_golden.py writes
the fixtures) and the GPU model (tests/test_forcing_rhs.py), so both see the
same arithmetic. Each builder returns the forcing function; patterns are
formed from the mesh at build time.
"""
import numpy as np


def buoyancy_rows(model, Q=0.05):
    """Heating of the bottom fluid row, uniform cooling above
    (forced_convection.py "RB" form)."""
    nh = model.param.halowidth
    ny = model.param.ny

    def forcing(param, mesh, s, ds):
        ds.b[nh, nh:-nh] += Q
        ds.b[nh + 1:-nh, nh:-nh] -= Q / (ny - 1)

    return forcing


def wind_curl(model, tau0=5e-3):
    """Constant curl of a zonal wind stress added to the PV tendency
    (gyre.py form), masked by msk and scaled by the cell area."""
    mesh = model.mesh
    Ly = model.param.Ly
    x, y = mesh.xy()
    ky = np.pi / Ly
    curltau = -tau0 * ky * np.cos(ky * y) * mesh.msk * mesh.area

    def forcing(param, mesh, s, ds):
        ds.pv[:, :] += curltau

    return forcing


def wave_maker(model, amp=0.5, period=0.3):
    """A Gaussian momentum source oscillating in time, added to u.y at every
    point (internalwave_maker.py form); reads mesh.time.t, so the model's
    time line must be attached as mesh.time."""
    mesh = model.mesh
    x, y = mesh.xy()
    omega = 2 * np.pi / period
    perturb = (np.exp(-((x - 0.5) ** 2 + (y - 0.5) ** 2) / (2 * 0.06 ** 2))
               * mesh.dx ** 2 / omega * mesh.msky * amp)

    def forcing(param, mesh, s, ds):
        ds.u.y[:, :] += perturb * np.sin(mesh.time.t * omega)

    return forcing


def periodic_mass_source(model, Q=2e-4):
    """A mass source/sink pattern periodic in x (its halo columns equal their
    interior copies), added to h of a channel, masked by msk."""
    mesh = model.mesh
    Lx, Ly = model.param.Lx, model.param.Ly
    x, y = mesh.xy()
    pattern = (Q * np.cos(2 * np.pi * x / Lx) * np.sin(np.pi * y / Ly)
               * mesh.msk * mesh.area)

    def forcing(param, mesh, s, ds):
        ds.h[:, :] += pattern

    return forcing


BUILDERS = {"buoyancy_rows": buoyancy_rows, "wind_curl": wind_curl,
            "wave_maker": wave_maker, "periodic_mass_source": periodic_mass_source}
