"""Differentiable eulerpsi rollouts: a ``torch.autograd.Function`` over the
discrete adjoint kernels of the library.

The reference (``src/fluids2d``) has no differentiation; the map
differentiated here is its time step - the SSP-RK3 stages of
``integrators.py:92-107`` applied to the eulerpsi right-hand side and
diagnostics of ``equations.py:73-86`` - with the time step held fixed::

    omega_T = rollout(model, omega_0, nsteps, dt, every=20)
    loss = some_function(omega_T)
    loss.backward()          # omega_0.grad = (d omega_T / d omega_0)^T dloss

``omega_0`` is an FP64 CUDA tensor of shape (ny+6, nx+6) (the model's array
layout, halo included). The forward pass keeps the vorticity every ``every``
steps on the device; the backward pass recomputes each segment from its
checkpoint while recording the stage states and face velocities, then runs
the adjoint RK3 steps backwards (hand-written adjoint kernels of the WENO-Z
flux divergence, of perpgrad and of the centre-to-vertex average, and the same
multigrid-preconditioned Poisson solve for the adjoint streamfunction). The
model may be FP64 or FP32 (FP32 stencils with the FP64-refined Poisson
solve); the adjoint arithmetic is FP64 either way.

Restrictions (the library refuses other cases with an error): eulerpsi,
closed (non-periodic) basin, ``weno`` or ``upwind`` fluxes.
"""
from __future__ import annotations

import ctypes

import torch

from ._lib import check, lib

__all__ = ["rollout", "Rollout"]


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class Rollout(torch.autograd.Function):
    """omega_T = Rollout.apply(omega_0, model, nsteps, dt, every)."""

    @staticmethod
    def forward(ctx, omega0, model, nsteps, dt, every):
        if not omega0.is_cuda or omega0.dtype != torch.float64:
            raise TypeError("omega0 must be an FP64 CUDA tensor")
        shape = (model.param.ny + 6, model.param.nx + 6)
        if tuple(omega0.shape) != shape:
            raise ValueError(f"omega0 must have shape {shape}")
        w0 = omega0.detach().contiguous()
        out = torch.empty_like(w0)
        model._push()  # pending host edits of the mesh-independent state
        # the library works on its own stream: order it after torch's work
        torch.cuda.current_stream().synchronize()
        L = lib()
        check(L.f2d_adjoint_forward(model._h, _ptr(w0), _ptr(out), int(nsteps),
                                    float(dt), int(every)))
        check(L.f2d_sync(model._h))
        model._device_state_changed()
        ctx.model = model
        return out

    @staticmethod
    def backward(ctx, gout):
        g = gout.detach().to(torch.float64).contiguous()
        gin = torch.empty_like(g)
        torch.cuda.current_stream().synchronize()
        L = lib()
        check(L.f2d_adjoint_backward(ctx.model._h, _ptr(g), _ptr(gin)))
        check(L.f2d_sync(ctx.model._h))
        ctx.model._device_state_changed()
        return gin, None, None, None, None


def rollout(model, omega0, nsteps, dt, every=20):
    """Run ``nsteps`` fixed-``dt`` RK3 steps of ``model`` from ``omega0``
    (differentiable w.r.t. ``omega0``); returns the final vorticity."""
    return Rollout.apply(omega0, model, nsteps, dt, every)
