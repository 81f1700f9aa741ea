"""Ensemble: many independent eulerpsi or qg models stepped together.

The reference runs one model at a time (``tools.run_twin_experiments``,
tools.py:29-49, steps two in lockstep). An Ensemble advances ``len(sizes)``
members with their own grid sizes and masks; every kernel is one launch for
all members, each member keeps its own CFL time step, time line and Poisson
convergence. Fields are exchanged per member with the reference's names and
(ny+6, nx+6) float64 layout.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib, ptr
from .param import Param


class Ensemble:
    def __init__(self, param: Param, sizes, masks=None):
        param.check()
        if param.model not in ("eulerpsi", "qg"):
            raise NotImplementedError("ensembles run the eulerpsi and qg models")
        self.param = param
        self.sizes = [(int(nx), int(ny)) for nx, ny in sizes]
        n = len(self.sizes)
        nxs = (ctypes.c_int * n)(*[s[0] for s in self.sizes])
        nys = (ctypes.c_int * n)(*[s[1] for s in self.sizes])
        self._masks = []
        mp = (ctypes.c_void_p * n)()
        for b in range(n):
            m = None if masks is None else masks[b]
            if m is not None:
                m = np.ascontiguousarray(m, dtype=np.int8)
                nx, ny = self.sizes[b]
                assert m.shape == (ny + 6, nx + 6)
                mp[b] = m.ctypes.data
            else:
                mp[b] = None
            self._masks.append(m)
        s = _lib.params_struct(param)
        h = ctypes.c_void_p()
        check(lib().f2d_ensemble_create(ctypes.byref(s), n, nxs, nys, mp,
                                        ctypes.byref(h)))
        self._h = h

    def __len__(self):
        return len(self.sizes)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().f2d_ensemble_destroy(h)
            except Exception:
                pass
            self._h = ctypes.c_void_p()

    def shape(self, b):
        nx, ny = self.sizes[b]
        return (ny + 6, nx + 6)

    def set_field(self, b, name, array):
        a = np.ascontiguousarray(array, dtype=np.float64)
        assert a.shape == self.shape(b)
        check(lib().f2d_ensemble_field_set(self._h, b, name.encode(), ptr(a)))

    def get_field(self, b, name):
        out = np.zeros(self.shape(b))
        check(lib().f2d_ensemble_field_get(self._h, b, name.encode(), ptr(out)))
        return out

    def packed_size(self):
        """Elements of the packed all-members layout."""
        return int(lib().f2d_ensemble_packed_size(self._h))

    def set_fields(self, name, arrays):
        """Field `name` of every member from a list of (ny+6, nx+6) arrays
        (or one packed float64 array), in one copy and one kernel."""
        packed = self._pack(arrays)
        check(lib().f2d_ensemble_fields_set(self._h, name.encode(), ptr(packed), 0))

    def get_fields(self, name):
        """Field `name` of every member as a list of (ny+6, nx+6) arrays."""
        packed = np.empty(self.packed_size())
        check(lib().f2d_ensemble_fields_get(self._h, name.encode(), ptr(packed), 0))
        out, k = [], 0
        for b in range(len(self.sizes)):
            ny, nx = self.shape(b)
            out.append(packed[k:k + ny * nx].reshape(ny, nx))
            k += ny * nx
        return out

    def _pack(self, arrays):
        if isinstance(arrays, np.ndarray) and arrays.ndim == 1:
            packed = np.ascontiguousarray(arrays, dtype=np.float64)
        else:
            packed = np.concatenate([np.ascontiguousarray(a, dtype=np.float64).ravel()
                                     for a in arrays])
        if packed.size != self.packed_size():
            raise ValueError("packed size does not match the ensemble")
        return packed

    def set_stream(self, stream_ptr):
        check(lib().f2d_ensemble_set_stream(self._h, ctypes.c_void_p(stream_ptr)))

    def diag(self):
        check(lib().f2d_ensemble_diag(self._h))

    def autotune(self, reps=3):
        """Pick the multigrid schedule (tile rows, sweeps per leg, inner
        tolerance) of the batched solver by timing each candidate's solve of
        the current state on the GPU (f2d_ensemble_autotune); the state is
        unchanged. Returns the chosen schedule."""
        th, nu = ctypes.c_int(), ctypes.c_int()
        tin, ms = ctypes.c_double(), ctypes.c_double()
        check(lib().f2d_ensemble_autotune(self._h, int(reps), ctypes.byref(th),
                                          ctypes.byref(nu), ctypes.byref(tin),
                                          ctypes.byref(ms)))
        return {"tile_rows": th.value, "sweeps": nu.value, "tol_in": tin.value,
                "ms_per_solve": ms.value}

    def set_schedule(self, tile_rows, sweeps, tol_in=1e-6):
        """Set the batched solver's multigrid schedule directly
        (f2d_ensemble_set_schedule)."""
        check(lib().f2d_ensemble_set_schedule(self._h, int(tile_rows), int(sweeps),
                                              float(tol_in)))

    def run(self, nsteps):
        check(lib().f2d_ensemble_run(self._h, int(nsteps)))

    def time(self, b):
        t, dt, ite = ctypes.c_double(), ctypes.c_double(), ctypes.c_int64()
        check(lib().f2d_ensemble_time_get(self._h, b, ctypes.byref(t),
                                          ctypes.byref(dt), ctypes.byref(ite)))
        return t.value, dt.value, ite.value

    def sync(self):
        check(lib().f2d_ensemble_sync(self._h))

    def stats(self):
        c, it, lp, ls, li = (ctypes.c_int64() for _ in range(5))
        check(lib().f2d_ensemble_stats(self._h, ctypes.byref(c), ctypes.byref(it),
                                       ctypes.byref(lp), ctypes.byref(ls),
                                       ctypes.byref(li)))
        r = ctypes.c_int64()
        check(lib().f2d_ensemble_refine_rounds(self._h, ctypes.byref(r)))
        return dict(cells=c.value, poisson_iters=it.value, loop_iters=lp.value,
                    launches_per_step=ls.value, launches_per_iter=li.value,
                    refine_rounds=r.value)
