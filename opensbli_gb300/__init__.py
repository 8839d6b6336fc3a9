"""GB300 (sm_103a) residual-and-update path for OpenSBLI problem definitions.

    from opensbli_gb300 import GB300Backend     # drop-in for OPSC(alg)
    from opensbli_gb300 import Solver, problems # direct use with BlockSpec objects
"""
from . import abi, problems  # noqa: F401
from .spec import BlockSpec  # noqa: F401


def __getattr__(name):
    if name == "Solver":
        from .solver import Solver
        return Solver
    if name == "GB300Backend":
        from .backend import GB300Backend
        return GB300Backend
    raise AttributeError(name)
