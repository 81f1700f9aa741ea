"""Host-side mesh construction of the CUDA library (no GPU needed).

``f2d_mesh_build`` must reproduce the reference's masks, slip coefficients,
stencil orders and vertex index bit for bit (golden fixtures from the
reference), and ``f2d_set_order`` must equal the oracle on random masks.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from fluids2d_gb300 import _lib
from fluids2d_gb300.param import Param
from oracle import oracle as O

G = np.load(os.path.join(GOLDEN, "mesh.npz"), allow_pickle=False)


def _noslip(text):
    """param.noslip from its fixture text: None, True, False or a list of
    side names such as "['left', 'top']"."""
    fixed = {"None": None, "True": True, "False": False}
    if text in fixed:
        return fixed[text]
    if text.startswith("[") and text.endswith("]"):
        return [w.strip().strip("'\"") for w in text[1:-1].split(",") if w.strip()]
    raise ValueError(f"unexpected noslip fixture value {text!r}")


def _param(case):
    nx, ny, xper, maxo = (int(v) for v in G[case + "/params"])
    p = Param()
    p.model = "rsw"
    p.nx, p.ny, p.xperiodic, p.maxorder = nx, ny, bool(xper), maxo
    p.noslip = _noslip(str(G[case + "/noslip"]))
    return p


@pytest.mark.parametrize("case", list(G["names"]))
def test_mesh_build_matches_reference(case):
    p = _param(case)
    d = _lib.mesh_build(p, G[case + "/msk"])
    for k in ("mskx", "msky", "mskv", "slipcoef", "ocx", "ocy", "ovx", "ovy",
              "okx", "oky"):
        np.testing.assert_array_equal(d[k], G[case + "/" + k], err_msg=k)
    np.testing.assert_array_equal(d["gv"], G[case + "/Gv"])


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("shift", [1, 37, -1, -37, 2])
def test_set_order_random(seed, shift):
    rng = np.random.default_rng(seed)
    m = (rng.uniform(size=37 * 29) < 0.7).astype(np.int8)
    for maxorder in (6, 5, 4, 2):
        o = np.zeros_like(m)
        _lib.check(_lib.lib().f2d_set_order(_lib.ptr(m), m.size, shift,
                                            maxorder, _lib.ptr(o)))
        np.testing.assert_array_equal(o, O.set_order(m, shift, maxorder))


def test_mesh_build_rejects_bad_params():
    p = Param()
    p.model = "eulerpsi"
    p.nx = p.ny = 16
    p.halowidth = 2
    with pytest.raises(_lib.F2DError):
        _lib.mesh_build(p, np.ones((20, 20), np.int8))
    p.halowidth = 3
    p.yperiodic = True
    with pytest.raises(_lib.F2DError):
        _lib.mesh_build(p, np.ones((22, 22), np.int8))
