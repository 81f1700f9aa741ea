"""Import the unmodified reference (pvthinker/Fluids2d) in this container.

The reference needs numba, netCDF4, matplotlib and PIL, none of which are
installed. This module registers stand-in modules for them before importing
``fluids2d`` from the reference source tree:

* ``numba.njit``/``numba.jit`` become the identity decorator, so the
  ``@njit`` kernels of ``src/fluids2d/weno.py`` run as plain Python floats
  (IEEE binary64, no FMA contraction, the same operation order);
* the plotting and NetCDF modules are empty shells (``model.run`` only touches
  them when ``animation``/``nhis`` are set, which the golden cases never do).

Only the golden-fixture generator imports this; it needs the reference tree
on disk and therefore runs only where that tree is present.
"""
import os
import sys
import types

# the reference's ``src`` directory (the one holding the ``fluids2d``
# package); required, no default
REFERENCE_SRC = os.environ.get("F2D_REFERENCE_SRC", "")


def _install_stubs():
    nb = types.ModuleType("numba")

    def njit(*a, **k):
        if a and callable(a[0]):
            return a[0]
        return lambda f: f

    nb.njit = njit
    nb.jit = njit
    nb.prange = range
    nb.set_num_threads = lambda n: None
    nb.config = types.SimpleNamespace(NUMBA_DEFAULT_NUM_THREADS=1)
    sys.modules["numba"] = nb
    for name in ["matplotlib", "matplotlib.pyplot", "mpl_toolkits",
                 "mpl_toolkits.axes_grid1", "netCDF4", "PIL"]:
        sys.modules[name] = types.ModuleType(name)
    sys.modules["matplotlib"].rc = lambda *a, **k: None
    sys.modules["mpl_toolkits.axes_grid1"].make_axes_locatable = None
    sys.modules["netCDF4"].Dataset = None
    sys.modules["PIL"].Image = None


def load_reference():
    """Return the reference ``fluids2d`` package (with stand-in modules)."""
    if not REFERENCE_SRC or not os.path.isdir(REFERENCE_SRC):
        raise RuntimeError(
            "set F2D_REFERENCE_SRC to the reference's src directory (the one "
            f"holding the fluids2d package); got {REFERENCE_SRC!r}")
    _install_stubs()
    if REFERENCE_SRC not in sys.path:
        sys.path.insert(0, REFERENCE_SRC)
    import fluids2d  # noqa: E402
    return fluids2d
