"""The integer-pipe binary64 <-> binary32 conversions (common.cuh:
f64_to_f32_rn, f32_to_f64) give the bits of the hardware conversions on the
GPU, for every class of input: normal values over the whole binary32 range
and beyond, exact ties between neighbouring binary32 values (round half to
even), binary32 subnormals and the underflow to zero, overflow to infinity,
signed zeros, infinities and NaN (compared as NaN)."""
import struct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from fluids2d_gb300._lib import lib  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _inputs64(rng):
    v = [rng.standard_normal(200000) * 10.0 ** rng.integers(-50, 50, 200000)]
    ex = np.arange(-160, 140, dtype=np.float64)
    for mant in (1.0, 1.5, 1.9999999, 1.0000000596046448, 1.0000001788139343):
        v.append(mant * 2.0 ** ex)
        v.append(-mant * 2.0 ** ex)
    a = (rng.standard_normal(20000) * 2.0 ** rng.integers(-149, 127, 20000)).astype(np.float32)
    b = np.nextafter(a, np.float32(np.inf))
    ok = np.isfinite(a) & np.isfinite(b)
    v.append((a[ok].astype(np.float64) + b[ok].astype(np.float64)) / 2)  # exact ties
    v.append(np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 3.4028235677973366e38,
                       3.4028236e38, 1e-46, 7e-46, 1.401298464324817e-45, 2.1e-45,
                       -2.1e-45, 5e-324, 1.7976931348623157e308]))
    return np.ascontiguousarray(np.concatenate(v))


def _inputs32(rng):
    bits = rng.integers(0, 2 ** 32, 400000, dtype=np.uint64).astype(np.uint32)
    special = np.array([0, 0x80000000, 1, 0x80000001, 0x7FFFFF, 0x400000, 0x7F7FFFFF,
                        0x7F800000, 0xFF800000, 0x7FC00000, 0x00800000], dtype=np.uint32)
    return np.ascontiguousarray(np.concatenate([bits, special]).view(np.float32))


def test_conversions_match_hardware():
    rng = np.random.default_rng(0)
    x64 = _inputs64(rng)
    x32 = _inputs32(rng)
    n64, n32 = x64.size, x32.size
    sw32 = np.empty(n64, np.float32)
    hw32 = np.empty(n64, np.float32)
    sw64 = np.empty(n32, np.float64)
    hw64 = np.empty(n32, np.float64)
    rc = lib().f2d_test_conversions(x64.ctypes.data, n64, sw32.ctypes.data, hw32.ctypes.data,
                                    x32.ctypes.data, n32, sw64.ctypes.data, hw64.ctypes.data)
    assert rc == 0
    nan = np.isnan(hw32)
    assert np.array_equal(np.isnan(sw32), nan)
    assert np.array_equal(sw32[~nan].view(np.uint32), hw32[~nan].view(np.uint32))
    nan = np.isnan(hw64)
    assert np.array_equal(np.isnan(sw64), nan)
    assert np.array_equal(sw64[~nan].view(np.uint64), hw64[~nan].view(np.uint64))
    # and numpy's IEEE conversions agree (a check of the test's inputs)
    with np.errstate(over="ignore"):
        ref = x64.astype(np.float32)
    fin = ~np.isnan(ref)
    assert np.array_equal(hw32[fin].view(np.uint32), ref[fin].view(np.uint32))
