"""Host-side logic of the Python mirror that needs no GPU: parameter checks,
the state layout with a tracer (states.py:22-34), the ctypes parameter
struct, and the file naming / attributes of the Bulk and history writers."""
import json

import numpy as np
import pytest

import fluids2d_gb300 as f2d
from fluids2d_gb300 import _lib, diagnostics
from fluids2d_gb300.model import _allocate_state, _flat_fields, _specs


def _param(**kw):
    p = f2d.Param()
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def test_tracer_is_the_last_prognostic_variable():
    # add_tracer_to_spec (states.py:31-34): prognostic + (tracer,), then the
    # remaining variables
    names, prog = _specs(_param(model="rsw", tracer="q"))
    assert prog == ("u", "h", "q")
    assert names == ("u", "h", "q", "U", "omega", "ke", "p", "flx", "pv")
    names, prog = _specs(_param(model="eulerpsi", tracer="c"))
    assert names[:2] == ("omega", "c") and prog == ("omega", "c")
    names, prog = _specs(_param(model="boussinesq"))
    assert prog == ("b", "u")


def test_tracer_field_maps_to_the_device_field():
    p = _param(model="eulerpsi", tracer="q")
    s = _allocate_state(p, (10, 12))
    flat = dict(_flat_fields(s, "q"))
    assert "tracer" in flat and "q" not in flat
    assert flat["tracer"] is s.q


@pytest.mark.parametrize("bad", ["omega", "U", 3])
def test_tracer_name_must_be_new(bad):
    with pytest.raises((ValueError, AssertionError)):
        _param(model="eulerpsi", tracer=bad).check()


def test_models_and_integrators_accepted():
    for model in ("eulerpsi", "rsw", "qg", "euler", "boussinesq", "qgrsw"):
        for integ in ("rk3", "ef", "enrk3", "LFRA"):
            _param(model=model, integrator=integ).check()
    _param(model="boussinesq", precision="fp32").check()  # FP32 stencils, FP64 solve
    with pytest.raises(NotImplementedError):
        _param(model="hydrostatic").check()


def test_params_struct_carries_integrator_gamma_tracer():
    s = _lib.params_struct(_param(model="qgrsw", integrator="LFRA", RAgamma=0.2,
                                  tracer="q"))
    assert s.model == 5 and s.integrator == 3
    assert s.ragamma == 0.2 and s.tracer == 1
    s = _lib.params_struct(_param(model="boussinesq"))
    assert s.model == 4 and s.integrator == 0 and s.tracer == 0
    assert abs(s.ragamma - 0.1) < 1e-15


def test_writer_file_names_and_attributes():
    assert diagnostics._npz_name("bulk.nc") == "bulk.npz"
    assert diagnostics._npz_name("history") == "history.npz"
    assert diagnostics._npz_name("out.npz") == "out.npz"
    atts = diagnostics.get_atts_from_param(_param(model="rsw", xperiodic=True))
    # io.py:40-48: bools as int, None as "None"
    assert atts["xperiodic"] == 1 and atts["tracer"] == "None"
    json.dumps(atts)


def test_bulk_records_file_roundtrip(tmp_path):
    # the .npz container of Bulk.write/read without a GPU model: the record
    # file format alone
    f = tmp_path / "bulk.npz"
    data = {n: np.arange(3.0) + k for k, n in enumerate(diagnostics.Bulk.variables)}
    np.savez(f, attrs=np.array("{}"), **data)
    assert diagnostics.get_number_of_records(str(f)) == 3
    assert diagnostics.get_number_of_records(str(tmp_path / "none.npz")) == 0
