"""The C-ABI library loads and exports every entry point that
include/*.h declares; the Python layer fails loudly where no GPU is present
(there is no CPU fallback)."""
import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT
from fluids2d_gb300 import _lib


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        with open(h) as f:
            src = f.read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names.update(re.findall(r"\b(f2d_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "f2d_model_create" in names and "f2d_poisson_solve" in names
    assert len(names) >= 25


@pytest.mark.parametrize("name", declared_functions())
def test_library_exports(name):
    L = ctypes.CDLL(_lib.library_path())
    assert hasattr(L, name), name


def test_abi_version_and_defaults():
    L = _lib.lib()
    assert L.f2d_abi_version() == 1
    p = _lib.Params()
    assert L.f2d_params_default(ctypes.byref(p)) == 0
    assert p.halowidth == 3 and p.maxorder == 6 and abs(p.cfl - 0.9) < 1e-15


def test_params_struct_matches_header_size():
    # f2d_params: 6 ints, 9 doubles, 7 ints, 1 double, 1 int, 7 reserved ints
    assert ctypes.sizeof(_lib.Params) % 8 == 0
    assert ctypes.sizeof(_lib.Params) >= 6 * 4 + 9 * 8 + 7 * 4 + 8 + 4 + 28


def test_model_create_fails_loudly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import fluids2d_gb300 as f2d
    p = f2d.Param()
    p.model = "eulerpsi"
    p.nx = p.ny = 16
    with pytest.raises(f2d.F2DError):
        f2d.Model(p)
