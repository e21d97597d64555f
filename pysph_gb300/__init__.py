"""pysph_gb300: the PySPH particle-step hot path on GB300 (sm_103a).

Drop-in for the reference's ``pysph.base`` / ``pysph.sph`` / ``pysph.solver``
APIs on the neighbour search, the SPHCalc pair loop (SPHRho, TaitEquation,
SPHPressureGradient, MonaghanArtificialVsicosity, XSPHCorrection,
MonaghanBoundaryForce, GravityForce, PositionStepping with the cubic spline)
and the Euler / RK2 integrators.  All arithmetic runs in the CUDA kernels of
``pysph_gb300/csrc`` (C ABI in ``include/pysph_gb300.h``).

Use ``import pysph_gb300.base.api as base`` etc. where PySPH code imports
``pysph.base.api``.
"""
import types as _types

__version__ = "0.1.0"


def api():
    """Namespace with ``base``, ``sph`` and ``solver`` API modules."""
    from .base import api as base
    from .solver import api as solver
    from .sph import api as sph
    return _types.SimpleNamespace(base=base, sph=sph, solver=solver)
