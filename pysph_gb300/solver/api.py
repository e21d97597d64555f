"""Names of ``pysph.solver.api`` on the GPU path."""
from .integrator import (EulerIntegrator, Integrator, LeapFrogIntegrator,  # noqa: F401
                         PredictorCorrectorIntegrator, RK2Integrator, RK4Integrator)
from .solver import Solver  # noqa: F401
from .sph_equation import SPHIntegration, SPHOperation  # noqa: F401

HAS_CL = False
