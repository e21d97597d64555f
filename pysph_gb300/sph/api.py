"""Names of ``pysph.sph.api`` (the reference's sph package) on the GPU path."""
from .sph_calc import SPHCalc  # noqa: F401
from .sph_func import (BeckerBoundaryForce, CSPHFunctionParticle, Function,  # noqa: F401
                       GravityForce, IdealGasEquation, MomentumEquation,
                       MonaghanArtificialVsicosity, MonaghanBoundaryForce,
                       MorrisViscosity, NBodyForce, PositionStepping, SPHDensityRate,
                       SPHFunction, SPHFunctionParticle, SPHPressureGradient, SPHRho,
                       TaitEquation, VectorForce, XSPHCorrection, XSPHDensityRate)
