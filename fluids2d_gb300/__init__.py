"""fluids2d_gb300: GB300-native time-stepping hot path of Fluids2d.

Drop-in counterparts of ``fluids2d.Param`` and ``fluids2d.Model`` for the
eulerpsi, rsw, qg, euler, boussinesq and qgrsw models (with an optional
passive tracer): WENO/upwind/centered/CWENO flux reconstruction on the
masked grid, the rk3/ef/enrk3/LFRA integrators and the masked 5-point
Poisson/Helmholtz solves run as hand-written CUDA kernels for sm_103a behind
the C ABI of ``include/fluids2d_gb300.h``.
"""
from .param import Param  # noqa: F401
from .model import Model  # noqa: F401
from . import tools  # noqa: F401
from . import operators  # noqa: F401
from . import diagnostics  # noqa: F401
from . import io  # noqa: F401
from .ensemble import Ensemble  # noqa: F401
from ._lib import F2DError  # noqa: F401
