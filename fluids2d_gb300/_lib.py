"""ctypes binding of the C ABI (include/fluids2d_gb300.h).

The shared library is built in-tree by ``fluids2d_gb300.build``; this module
loads it and raises if it is missing. There is no CPU fallback: every compute
call goes through the CUDA library.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

c_int = ctypes.c_int
c_i64 = ctypes.c_int64
c_dbl = ctypes.c_double
c_void_p = ctypes.c_void_p

MODELS = {"eulerpsi": 0, "rsw": 1, "qg": 2, "euler": 3, "boussinesq": 4, "qgrsw": 5}
METHODS = {"weno": 0, "upwind": 1, "centered": 2, "cweno": 3}
PRECISIONS = {"fp64": 0, "fp32": 1}
INTEGRATORS = {"rk3": 0, "ef": 1, "enrk3": 2, "LFRA": 3}
SIDES = {"left": 1, "right": 2, "bottom": 4, "top": 8}


class F2DError(RuntimeError):
    """An error reported by the CUDA library (f2d_last_error)."""


class Params(ctypes.Structure):
    _fields_ = [
        ("model", c_int), ("nx", c_int), ("ny", c_int), ("halowidth", c_int),
        ("xperiodic", c_int), ("yperiodic", c_int),
        ("Lx", c_dbl), ("Ly", c_dbl),
        ("f0", c_dbl), ("beta", c_dbl), ("g", c_dbl), ("H", c_dbl),
        ("cfl", c_dbl), ("dtmax", c_dbl), ("dt", c_dbl),
        ("compflux", c_int), ("vortexforce", c_int), ("innerproduct", c_int),
        ("maxorder", c_int), ("noslip", c_int), ("noslip_sides", c_int),
        ("precision", c_int),
        ("poisson_tol", c_dbl), ("poisson_maxit", c_int),
        ("integrator", c_int),
        ("ragamma", c_dbl),
        ("tracer", c_int),
        ("reserved", c_int * 3),
    ]


_LIB = None

_SIGS = {
    "f2d_abi_version": ([], c_int),
    "f2d_last_error": ([], ctypes.c_char_p),
    "f2d_params_default": ([ctypes.POINTER(Params)], c_int),
    "f2d_set_order": ([c_void_p, c_i64, c_i64, c_int, c_void_p], c_int),
    "f2d_mesh_build": ([ctypes.POINTER(Params), c_void_p, c_void_p, c_void_p,
                        c_void_p, c_void_p, c_void_p, c_void_p], c_int),
    "f2d_compflux": ([c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_i64,
                      c_i64, c_i64, c_void_p], c_int),
    "f2d_vortexforce": ([c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_i64,
                         c_i64, c_int, c_i64, c_i64, c_void_p], c_int),
    "f2d_innerproduct": ([c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                          c_i64, c_i64, c_i64, c_void_p], c_int),
    "f2d_model_create": ([ctypes.POINTER(Params), c_void_p,
                          ctypes.POINTER(c_void_p)], c_int),
    "f2d_model_destroy": ([c_void_p], c_int),
    "f2d_model_set_mask": ([c_void_p, c_void_p], c_int),
    "f2d_model_set_stream": ([c_void_p, c_void_p], c_int),
    "f2d_field_set": ([c_void_p, ctypes.c_char_p, c_void_p], c_int),
    "f2d_field_get": ([c_void_p, ctypes.c_char_p, c_void_p], c_int),
    "f2d_field_set_async": ([c_void_p, ctypes.c_char_p, c_void_p], c_int),
    "f2d_field_get_async": ([c_void_p, ctypes.c_char_p, c_void_p], c_int),
    "f2d_field_device": ([c_void_p, ctypes.c_char_p, ctypes.POINTER(c_void_p),
                          ctypes.POINTER(c_i64), ctypes.POINTER(c_int)], c_int),
    "f2d_field_names": ([c_void_p, ctypes.c_char_p, ctypes.c_size_t], c_int),
    "f2d_set_coriolis": ([c_void_p, c_void_p], c_int),
    "f2d_diag": ([c_void_p], c_int),
    "f2d_qg_projection": ([c_void_p], c_int),
    "f2d_field_get_f32": ([c_void_p, ctypes.c_char_p, c_void_p], c_int),
    "f2d_bulk_record": ([c_void_p], c_int),
    "f2d_ensemble_fields_set": ([c_void_p, ctypes.c_char_p, c_void_p, c_int], c_int),
    "f2d_ensemble_fields_get": ([c_void_p, ctypes.c_char_p, c_void_p, c_int], c_int),
    "f2d_ensemble_packed_size": ([c_void_p], ctypes.c_int64),
    "f2d_autotune": ([c_void_p, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int),
                      ctypes.POINTER(c_dbl), ctypes.POINTER(c_dbl)], c_int),
    "f2d_ensemble_autotune": ([c_void_p, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int),
                               ctypes.POINTER(c_dbl), ctypes.POINTER(c_dbl)], c_int),
    "f2d_bulk_read": ([c_void_p, c_void_p, c_int, ctypes.POINTER(c_int)], c_int),
    "f2d_step": ([c_void_p, c_int], c_int),
    "f2d_run": ([c_void_p, c_int], c_int),
    "f2d_set_dt": ([c_void_p], c_int),
    "f2d_time_get": ([c_void_p, ctypes.POINTER(c_dbl), ctypes.POINTER(c_dbl),
                      ctypes.POINTER(c_i64)], c_int),
    "f2d_time_set": ([c_void_p, c_dbl, c_dbl, c_i64], c_int),
    "f2d_poisson_solve": ([c_void_p, c_int, c_void_p, c_void_p,
                           ctypes.POINTER(c_int), ctypes.POINTER(c_dbl)], c_int),
    "f2d_sync": ([c_void_p], c_int),
    "f2d_time_stage": ([c_void_p, c_int, c_int, c_int, ctypes.POINTER(c_dbl)],
                       c_int),
    "f2d_ensemble_create": ([ctypes.POINTER(Params), c_int, c_void_p, c_void_p,
                             c_void_p, ctypes.POINTER(c_void_p)], c_int),
    "f2d_ensemble_destroy": ([c_void_p], c_int),
    "f2d_ensemble_set_stream": ([c_void_p, c_void_p], c_int),
    "f2d_ensemble_field_set": ([c_void_p, c_int, ctypes.c_char_p, c_void_p], c_int),
    "f2d_ensemble_field_get": ([c_void_p, c_int, ctypes.c_char_p, c_void_p], c_int),
    "f2d_ensemble_field_set_async": ([c_void_p, c_int, ctypes.c_char_p, c_void_p],
                                     c_int),
    "f2d_ensemble_field_get_async": ([c_void_p, c_int, ctypes.c_char_p, c_void_p],
                                     c_int),
    "f2d_ensemble_diag": ([c_void_p], c_int),
    "f2d_ensemble_run": ([c_void_p, c_int], c_int),
    "f2d_ensemble_time_get": ([c_void_p, c_int, ctypes.POINTER(c_dbl),
                               ctypes.POINTER(c_dbl), ctypes.POINTER(c_i64)], c_int),
    "f2d_ensemble_sync": ([c_void_p], c_int),
    "f2d_ensemble_stats": ([c_void_p] + [ctypes.POINTER(c_i64)] * 5, c_int),
    "f2d_ensemble_time_stage": ([c_void_p, c_int, c_int, c_int,
                                 ctypes.POINTER(c_dbl)], c_int),
    "f2d_time_solver": ([c_void_p, c_int, c_int, ctypes.POINTER(c_dbl),
                         ctypes.POINTER(c_i64), ctypes.POINTER(c_int)], c_int),
    "f2d_ensemble_time_solver": ([c_void_p, c_int, c_int, ctypes.POINTER(c_dbl),
                                  ctypes.POINTER(c_i64), ctypes.POINTER(c_int)], c_int),
    "f2d_solver_pipelined": ([c_void_p, ctypes.POINTER(c_int)], c_int),
    "f2d_ensemble_solver_pipelined": ([c_void_p, ctypes.POINTER(c_int)], c_int),
    "f2d_adjoint_forward": ([c_void_p, c_void_p, c_void_p, c_int, c_dbl, c_int], c_int),
    "f2d_adjoint_backward": ([c_void_p, c_void_p, c_void_p], c_int),
    "f2d_cfl_dt_noalloc": ([c_void_p, c_void_p, c_i64, c_i64, c_i64, c_dbl,
                            c_dbl, c_void_p, c_void_p], c_int),
    "f2d_stats": ([c_void_p, ctypes.POINTER(c_i64), ctypes.POINTER(c_i64),
                   ctypes.POINTER(c_i64)], c_int),
    "f2d_test_tma_wait": ([c_int, c_dbl], c_int),
    "f2d_test_conversions": ([c_void_p, c_i64, c_void_p, c_void_p, c_void_p, c_i64,
                              c_void_p, c_void_p], c_int),
    "f2d_rhs": ([c_void_p], c_int),
    "f2d_set_schedule": ([c_void_p, c_int, c_int, c_dbl], c_int),
    "f2d_ensemble_set_schedule": ([c_void_p, c_int, c_int, c_dbl], c_int),
    "f2d_refine_rounds": ([c_void_p, ctypes.POINTER(c_i64)], c_int),
    "f2d_ensemble_refine_rounds": ([c_void_p, ctypes.POINTER(c_i64)], c_int),
    "f2d_stage": ([c_void_p, c_int], c_int),
    "f2d_forcing_set": ([c_void_p, ctypes.c_char_p, c_void_p], c_int),
    "f2d_forcing_clear": ([c_void_p], c_int),
}


def library_path():
    return _build.LIB


def lib():
    """Load the CUDA library (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        path = _build.LIB
        if not os.path.exists(path):
            raise F2DError(
                f"CUDA library not built: {path} is missing; run "
                "fluids2d_gb300.build.build() (or __graft_entry__.build())")
        L = ctypes.CDLL(path)
        for name, (args, res) in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _LIB = L
    return _LIB


def check(rc):
    if rc != 0:
        msg = lib().f2d_last_error()
        raise F2DError(f"[{rc}] {msg.decode() if msg else 'unknown error'}")
    return rc


def ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def params_struct(p):
    """Fill a Params struct from a fluids2d_gb300.Param."""
    s = Params()
    check(lib().f2d_params_default(ctypes.byref(s)))
    s.model = MODELS[p.model]
    s.nx, s.ny = int(p.nx), int(p.ny)
    s.halowidth = int(p.halowidth)
    s.xperiodic = int(bool(p.xperiodic))
    s.yperiodic = int(bool(p.yperiodic))
    s.Lx, s.Ly = float(p.Lx), float(p.Ly)
    s.f0, s.beta = float(p.f0), float(p.beta)
    s.g, s.H = float(p.g), float(p.H)
    s.cfl, s.dtmax, s.dt = float(p.cfl), float(p.dtmax), float(p.dt)
    s.compflux = METHODS[p.compflux]
    s.vortexforce = METHODS[p.vortexforce]
    ip = p.innerproduct
    s.innerproduct = 4 if ip == "classic" else METHODS[ip]
    s.maxorder = int(p.maxorder)
    ns = p.noslip
    if ns is None or ns is False:
        s.noslip, s.noslip_sides = 0, 0
    elif ns is True:
        s.noslip, s.noslip_sides = 1, 0
    else:
        s.noslip = 2
        s.noslip_sides = sum(v for k, v in SIDES.items() if k in ns)
    s.precision = PRECISIONS[getattr(p, "precision", "fp64")]
    s.poisson_tol = float(getattr(p, "poisson_tol", 1e-12))
    s.poisson_maxit = int(getattr(p, "poisson_maxit", 200))
    s.integrator = INTEGRATORS[getattr(p, "integrator", "rk3")]
    s.ragamma = float(getattr(p, "RAgamma", 0.1))
    tr = getattr(p, "tracer", None)
    s.tracer = 0 if tr is None or tr == "None" else 1
    return s


def mesh_build(p, msk):
    """Host-side masks/orders/index (f2d_mesh_build)."""
    s = params_struct(p)
    msk = np.ascontiguousarray(msk, dtype=np.int8)
    shape = msk.shape
    mskx = np.zeros(shape, np.int8)
    msky = np.zeros(shape, np.int8)
    mskv = np.zeros(shape, np.int8)
    slip = np.zeros(shape, np.float64)
    orders = np.zeros((6,) + shape, np.int8)
    gv = np.zeros(shape, np.int32)
    check(lib().f2d_mesh_build(ctypes.byref(s), ptr(msk), ptr(mskx), ptr(msky),
                               ptr(mskv), ptr(slip), ptr(orders), ptr(gv)))
    return dict(mskx=mskx, msky=msky, mskv=mskv, slipcoef=slip,
                ocx=orders[0], ocy=orders[1], ovx=orders[2], ovy=orders[3],
                okx=orders[4], oky=orders[5], gv=gv)
