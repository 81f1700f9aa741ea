"""tools.set_uv_from_omega (tools.py:6-26 of the reference): velocity from a
vertex vorticity through the vertex Poisson solve and perpgrad."""
import numpy as np


def set_uv_from_omega(model, omega, u, contravariant=False):
    mesh = model.mesh
    psi = omega * 0
    mesh.poisson_vertices.solve(omega, psi)
    u.x[:-1, :] = -np.diff(psi, axis=0) * mesh.mskx[:-1, :]
    u.y[:, :-1] = np.diff(psi, axis=1) * mesh.msky[:, :-1]
    if contravariant:
        u.x[:] *= (1 / mesh.dy ** 2)
        u.y[:] *= (1 / mesh.dx ** 2)
