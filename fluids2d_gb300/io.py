"""History output: the counterpart of the reference's ``fluids2d.io.IO``
(io.py:5-92).

Every ``param.nhis`` iterations (timeline.py:47-51) ``Model.run`` stores
``t``, ``ite``, ``dt`` and the fields of ``param.var_to_store`` as float32
(the reference's dtype "f"; converted on the GPU by ``f2d_field_get_f32``,
half the bytes of the FP64 state cross to the host). netCDF4 is not
available to this package: the records are kept in host memory and written
as a NumPy ``.npz`` with the reference's variable names (vectors as
``<name>x``, ``<name>y``; ``xc``, ``yc``; parameters as JSON ``attrs``); the
``.nc`` suffix of ``param.outputfile`` becomes ``.npz``.
"""
from __future__ import annotations

import json

import numpy as np

from ._lib import check, lib, ptr
from .diagnostics import _npz_name, get_atts_from_param

VECTORS = ("u", "U", "flx", "v")


class IO:
    """io.py:5-21."""

    def __init__(self, param, mesh, state, time):
        self.param = param
        self.mesh = mesh
        self.kt = 0
        self.records = {"t": [], "ite": [], "dt": []}
        self.file = _npz_name(param.outputfile)
        if param.nhis > 0:
            self.create_file()

    def create_file(self):
        """io.py:51-92: coordinates and the empty record lists."""
        x, y = self.mesh.xy()
        self.xc = x.astype(np.float32)
        self.yc = y.astype(np.float32)
        for name in self.param.var_to_store:
            if name in VECTORS:
                self.records[name + "x"] = []
                self.records[name + "y"] = []
            else:
                self.records[name] = []
        self.flush()

    def _get_f32(self, model, device_name):
        out = np.empty(self.mesh.shape, dtype=np.float32)
        check(lib().f2d_field_get_f32(model._h, device_name.encode(), ptr(out)))
        return out

    def write(self, model):
        """io.py:12-21 for the model's current state."""
        t, dt, ite = model.time._get()
        self.records["t"].append(np.float32(t))
        self.records["ite"].append(np.int32(ite))
        self.records["dt"].append(np.float32(dt))
        tracer = getattr(model, "_tracer", None)
        for name in self.param.var_to_store:
            if name in VECTORS:
                self.records[name + "x"].append(self._get_f32(model, name + ".x"))
                self.records[name + "y"].append(self._get_f32(model, name + ".y"))
            else:
                dev = "tracer" if name == tracer else name
                self.records[name].append(self._get_f32(model, dev))
        self.kt += 1

    def flush(self):
        data = {k: np.array(v) for k, v in self.records.items()}
        np.savez(self.file, attrs=np.array(json.dumps(get_atts_from_param(self.param))),
                 xc=self.xc, yc=self.yc, **data)
