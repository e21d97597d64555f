"""Names of ``pysph.sph.api`` (the reference's sph package) on the GPU path."""
from .sph_calc import SPHCalc  # noqa: F401
from .sph_func import (ADKEConductionCoeffUpdate, ADKEPilotRho,  # noqa: F401
                       ADKESmoothingUpdate, BeckerBoundaryForce, CSPHFunctionParticle, Function,
                       GravityForce, IdealGasEquation, MomentumEquation,
                       MonaghanArtificialVsicosity, MonaghanBoundaryForce,
                       MorrisViscosity, NBodyForce, PositionStepping, SPHDensityRate,
                       SPHFunction, SPHFunctionParticle, SPHPressureGradient, SPHRho,
                       SPHVelocityDivergence, TaitEquation, VectorForce, VelocityDivergence,
                       XSPHCorrection, XSPHDensityRate)
