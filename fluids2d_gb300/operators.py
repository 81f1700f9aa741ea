"""Operators of the reference's ``fluids2d.operators`` that user code calls
on a model's state (operators.py), executed on the GPU for a model of this
package."""
from __future__ import annotations


def qg_projection(mesh, u, h, pv, psi, anomaly=False):
    """operators.py:176-183: project (u, h) on the QG manifold.

    ``mesh`` is the ``Mesh`` of a qgrsw ``Model`` of this package and u, h,
    pv, psi are that model's state fields (``model.state.u`` ...); the
    projection runs on the GPU and the state is updated in place. The
    anomaly=True form is the tendency projection inside the qgrsw right-hand
    side and is not a user entry point.
    """
    m = getattr(mesh, "_m", None)
    if m is None:
        raise TypeError("mesh must be the Mesh of a fluids2d_gb300 Model")
    if anomaly:
        raise NotImplementedError("anomaly=True is the qgrsw tendency projection; "
                                  "it runs inside the model's step")
    s = m._state
    if not (u is s.u and h is s.h and pv is s.pv and psi is s.psi):
        raise ValueError("u, h, pv, psi must be the model's own state fields")
    m.qg_projection()
