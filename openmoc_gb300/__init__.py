"""GB300 (sm_103a) method-of-characteristics transport solver with
OpenMOC's Solver interface.

    from openmoc_gb300 import GB300Solver
    solver = GB300Solver(problem)          # packed tracks + cross sections
    solver.setConvergenceThreshold(1e-5)
    solver.computeEigenvalue()
    solver.getKeff(), solver.getFlux(fsr, group)
"""
from .cmfd import Cmfd  # noqa: F401
from .problem import Problem, instances, load_packed, save_packed  # noqa: F401
from .solver import (EXP_INTRINSIC, EXP_TABLE, FISSION_SOURCE,  # noqa: F401
                     SCALAR_FLUX, TOTAL_SOURCE, GB300LSSolver, GB300Solver)

__all__ = ["GB300Solver", "GB300LSSolver", "Cmfd", "Problem", "load_packed", "save_packed",
           "SCALAR_FLUX", "FISSION_SOURCE", "TOTAL_SOURCE", "EXP_TABLE",
           "EXP_INTRINSIC"]
