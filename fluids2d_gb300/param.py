"""Param: the reference's parameter bag (pvthinker/Fluids2d, param.py).

Same attribute names, defaults and checks (unknown attributes are refused by
``check``, enum values are asserted). Three knobs are added for this
implementation and listed in ``EXTRA``: ``precision`` ("fp64" or "fp32"),
``poisson_tol`` (relative residual of the multigrid-PCG solve) and
``poisson_maxit``.
"""

_models = ["euler", "eulerpsi", "advection", "vectoradv",
           "boussinesq", "hydrostatic", "rsw", "qgrsw", "qg"]
_methods = ["weno", "upwind", "centered", "cweno"]
_methods_extended = _methods + ["classic"]
_integrators = ["rk3", "ef", "enrk3", "LFRA"]

# models and integrators the GPU path implements
SUPPORTED_MODELS = ("eulerpsi", "rsw", "qg", "euler", "boussinesq", "qgrsw")
# the state variables of those models (states.py:7-17)
MODEL_VARIABLES = {
    "eulerpsi": ("omega", "U", "psi", "vomega", "flx"),
    "euler": ("u", "U", "omega", "ke", "p", "div", "flx"),
    "boussinesq": ("b", "u", "U", "omega", "ke", "p", "div", "flx"),
    "rsw": ("u", "h", "U", "omega", "ke", "p", "flx", "pv"),
    "qg": ("pv", "U", "h", "flx", "work", "psi"),
    "qgrsw": ("u", "h", "U", "omega", "ke", "p", "flx", "pv", "psi"),
}
SUPPORTED_INTEGRATORS = ("rk3", "ef", "enrk3", "LFRA")
EXTRA = ("precision", "poisson_tol", "poisson_maxit")


class Param:
    def __init__(self):
        self.model = "euler"
        self.nx = 40
        self.ny = 40
        self.Lx = 1.0
        self.Ly = 1.0
        self.xperiodic = False
        self.yperiodic = False
        self.halowidth = 3
        self.noslip = None
        self.f0 = 10.0
        self.beta = 0.0
        self.g = 1
        self.H = 1
        self.tend = 1.0
        self.dt = 0.0
        self.maxite = 100
        self.dtmax = 9e99
        self.nprint = 1
        self.nplot = 5
        self.animation = False
        self.generate_mp4 = False
        self.plotvar = None
        self.clims = None
        self.cmap = "RdBu_r"
        self.outputfile = "history.nc"
        self.var_to_store = []
        self.nhis = 0
        self.integrator = "rk3"
        self.cfl = 0.9
        self.RAgamma = 0.1
        self.compflux = "weno"
        self.vortexforce = "weno"
        self.innerproduct = "weno"
        self.maxorder = 6
        self.tracer = None
        self.nthreads = 1
        # additions of this implementation
        self.precision = "fp64"
        self.poisson_tol = 1e-12
        self.poisson_maxit = 200
        self.__parameters__ = _parameters(self)

    def add_parameter(self, name):
        """param.py:64-66."""
        setattr(self, name, None)
        self.__parameters__ = _parameters(self)

    def check_parameters_are_known(self):
        """param.py:68-75."""
        extra = set(_parameters(self)).difference(set(self.__parameters__))
        if extra:
            raise AssertionError(f"parameter {extra} is unknown\n"
                                 f"parameters are {self.__parameters__}")
        return True

    def check(self):
        """param.py:77-87, plus the limits of the GPU path."""
        assert self.model in _models
        assert self.compflux in _methods
        assert self.vortexforce in _methods
        assert self.innerproduct in _methods_extended
        assert self.integrator in _integrators
        self.check_parameters_are_known()
        if self.model not in SUPPORTED_MODELS:
            raise NotImplementedError(
                f"model {self.model!r}: the GPU path implements "
                f"{', '.join(SUPPORTED_MODELS)}")
        if self.integrator not in SUPPORTED_INTEGRATORS:
            raise NotImplementedError(
                f"integrator {self.integrator!r}: the GPU path implements "
                f"{', '.join(SUPPORTED_INTEGRATORS)}")
        if self.tracer not in (None, "None"):
            names = MODEL_VARIABLES.get(self.model, ())
            if not isinstance(self.tracer, str) or self.tracer in names:
                raise ValueError(f"tracer name {self.tracer!r} must be a new "
                                 "state variable name")
        if self.halowidth != 3:
            raise NotImplementedError("halowidth must be 3")
        if self.yperiodic:
            raise NotImplementedError("yperiodic is not supported")
        assert self.precision in ("fp64", "fp32")


def _parameters(obj):
    return [d for d in obj.__dir__() if "__" not in d]
