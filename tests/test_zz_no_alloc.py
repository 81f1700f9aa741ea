"""The allocation-free CFL entry point, f2d_cfl_dt_noalloc, against the
model's own set_dt.

Callers that cannot allocate device memory (frameworks that route all device
memory through their own pool, loops where a cudaMalloc would synchronise the
device) use f2d_cfl_dt_noalloc with their own device arrays; it must give the same max|U| and time step as the existing
path (f2d_field_set -> f2d_set_dt -> f2d_time_get), call after call, although
its scratch array is shared and reused. Tolerance: 1e-10 relative, as in the
other GPU parity tests (a maximum is exact, so equality is expected).

This file is collected last, so a run that stops at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import fluids2d_gb300 as f2d  # noqa: E402
from fluids2d_gb300._lib import check, lib  # noqa: E402

TOL = 1e-10


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _model(n=96, ny=80):
    p = f2d.Param()
    p.model = "eulerpsi"
    p.nx, p.ny = n, ny
    p.cfl = 0.8
    return f2d.Model(p)


def _device(m, name):
    ptr, pitch, es = ctypes.c_void_p(), ctypes.c_int64(), ctypes.c_int()
    check(lib().f2d_field_device(m._h, name.encode(), ctypes.byref(ptr),
                                 ctypes.byref(pitch), ctypes.byref(es)))
    return ptr, pitch.value


def _existing_dt(m, ux, uy):
    """The existing path: upload U from the host, set_dt on the device."""
    for name, a in (("U.x", ux), ("U.y", uy)):
        a = np.ascontiguousarray(a)
        check(lib().f2d_field_set(m._h, name.encode(),
                                  ctypes.c_void_p(a.ctypes.data)))
    check(lib().f2d_set_dt(m._h))
    dt = ctypes.c_double()
    check(lib().f2d_time_get(m._h, None, ctypes.byref(dt), None))
    return dt.value


def test_noalloc_cfl_matches_set_dt_twice():
    m = _model()
    shape = m.mesh.shape
    rows, cols = shape
    pux, pitch = _device(m, "U.x")
    puy, _ = _device(m, "U.y")
    out = torch.full((3,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(123)
    for call, scale in enumerate((1.0, 1e-3)):
        ux = rng.normal(size=shape) * scale
        uy = rng.normal(size=shape) * scale * 2.5
        dt_ref = _existing_dt(m, ux, uy)  # also leaves ux, uy on the device
        check(lib().f2d_cfl_dt_noalloc(pux, puy, rows, cols, pitch, 0.8, 9e99,
                                       ctypes.c_void_p(out.data_ptr()),
                                       ctypes.c_void_p(stream)))
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert abs(got[0] - np.max(np.abs(ux))) <= TOL * np.max(np.abs(ux))
        assert abs(got[1] - np.max(np.abs(uy))) <= TOL * np.max(np.abs(uy))
        assert abs(got[2] - dt_ref) <= TOL * dt_ref, (call, got[2], dt_ref)
    m.sync()


def test_noalloc_cfl_dtmax_and_size_limit():
    m = _model(64, 64)
    rows, cols = m.mesh.shape
    pux, pitch = _device(m, "U.x")
    puy, _ = _device(m, "U.y")
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    z = np.zeros(m.mesh.shape)
    _existing_dt(m, z, z)
    check(lib().f2d_cfl_dt_noalloc(pux, puy, rows, cols, pitch, 0.8, 0.125,
                                   ctypes.c_void_p(out.data_ptr()), None))
    torch.cuda.synchronize()
    assert out[2].item() == 0.125  # U = 0: the dtmax cap
    # beyond the fixed scratch: refused before any device work
    rc = lib().f2d_cfl_dt_noalloc(pux, puy, 40000, cols, 1000, 0.8, 1.0,
                                  ctypes.c_void_p(out.data_ptr()), None)
    assert rc != 0
    assert b"too large" in lib().f2d_last_error()


def test_noalloc_cfl_propagates_nan_like_set_dt():
    """A NaN in U gives NaN maxima and a NaN time step, as np.max and min()
    give in the reference's set_dt (model.py:83-87), and as the model's own
    set_dt gives; a finite U afterwards gives finite values again."""
    m = _model(64, 48)
    rows, cols = m.mesh.shape
    pux, pitch = _device(m, "U.x")
    puy, _ = _device(m, "U.y")
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    rng = np.random.default_rng(7)
    ux = rng.normal(size=m.mesh.shape)
    uy = rng.normal(size=m.mesh.shape)
    ux[10, 11] = np.nan
    dt_ref = _existing_dt(m, ux, uy)
    assert np.isnan(dt_ref)
    with pytest.raises(f2d.F2DError, match="non-finite"):
        m.sync()
    check(lib().f2d_cfl_dt_noalloc(pux, puy, rows, cols, pitch, 0.8, 9e99,
                                   ctypes.c_void_p(out.data_ptr()), None))
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert np.isnan(got[0]) and not np.isnan(got[1]) and np.isnan(got[2])
    ux[10, 11] = 0.0
    dt_ref = _existing_dt(m, ux, uy)
    check(lib().f2d_cfl_dt_noalloc(pux, puy, rows, cols, pitch, 0.8, 9e99,
                                   ctypes.c_void_p(out.data_ptr()), None))
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert np.isfinite(got).all() and abs(got[2] - dt_ref) <= TOL * dt_ref
    m.sync()
