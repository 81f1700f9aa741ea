"""Bulk diagnostics: the counterpart of the reference's ``fluids2d.diagnostics
.Bulk`` (diagnostics.py:8-80).

Every third iteration (diagnostics.py:40) the domain averages of the
current state - kinetic energy, enstrophy, vorticity, angular momentum - are
reduced on the GPU and appended to a device ring (``f2d_bulk_record``): no
host synchronisation per record. ``write()`` (every ``ndiags`` records and at
``finalize()``) drains the ring and appends the records to ``ncfile``.
netCDF4 is not available to this package, so the file is a NumPy ``.npz``
with the reference's variable names (``time, ke, ens, vort, angular``) and
the parameters as attributes (JSON in ``attrs``); the name's ``.nc`` suffix
becomes ``.npz``.
"""
from __future__ import annotations

import ctypes
import json
import os
from collections import namedtuple

import numpy as np

from ._lib import check, lib, ptr


def _npz_name(name):
    root, ext = os.path.splitext(name)
    return root + ".npz" if ext in (".nc", "") else name


def get_atts_from_param(param):
    """io.py:40-48: the parameters as attributes (bools as int, None as
    "None")."""
    atts = {}
    for k, v in param.__dict__.items():
        if k.startswith("_"):
            continue
        v = int(v) if isinstance(v, bool) else v
        v = "None" if v is None else v
        try:
            json.dumps(v)
        except TypeError:
            v = str(v)
        atts[k] = v
    return atts


class Bulk:
    """diagnostics.py:8-71 (``model.diags.append(Bulk(model))``)."""

    variables = ("time", "ke", "ens", "vort", "angular")

    def __init__(self, model, ncfile="bulk.nc"):
        self.model = model
        self.Bulk = namedtuple("bulk", self.variables)
        self.ndiags = 1_000
        self.kt = 0
        self.ncfile = _npz_name(ncfile)
        self.k0 = get_number_of_records(self.ncfile)
        if self.k0 == 0:
            self.create_newfile()

    def create_newfile(self):
        self._save({name: np.zeros((0,)) for name in self.variables})
        self.k0 = 0

    def __call__(self):
        if self.model.time.ite % 3 > 0:
            return
        m = self.model
        m._push()
        check(lib().f2d_bulk_record(m._h))
        self.kt += 1
        if self.kt == self.ndiags:
            self.write()

    def finalize(self):
        self.write()

    def records(self):
        """Drain the device ring: (n, 5) array of time, ke, ens, vort,
        angular."""
        buf = np.zeros((self.ndiags, 5))
        n = ctypes.c_int(0)
        check(lib().f2d_bulk_read(self.model._h, ptr(buf), self.ndiags,
                                  ctypes.byref(n)))
        return buf[:n.value]

    def write(self):
        rec = self.records()
        old = self.read()
        data = {name: np.concatenate([getattr(old, name), rec[:, k]])
                for k, name in enumerate(self.variables)}
        self._save(data)
        self.k0 += len(rec)
        self.kt = 0

    def read(self):
        with np.load(self.ncfile) as f:
            return self.Bulk(*[f[name] for name in self.variables])

    def _save(self, data):
        attrs = json.dumps(get_atts_from_param(self.model.param))
        np.savez(self.ncfile, attrs=np.array(attrs), **data)


def get_number_of_records(ncfile):
    """diagnostics.py:100-106."""
    if os.path.isfile(ncfile):
        with np.load(ncfile) as f:
            return len(f["time"])
    return 0
