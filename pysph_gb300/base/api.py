"""Names of ``pysph.base.api`` (the reference's base package)."""
from .carray import DoubleArray, FloatArray, IntArray, LongArray  # noqa: F401
from .cell import CellManager, PeriodicDomain  # noqa: F401
from .kernels import (CubicSplineKernel, DummyKernel, GaussianKernel,  # noqa: F401
                      HarmonicKernel, KernelBase, M6SplineKernel, Poly6Kernel,
                      QuinticSplineKernel, W8Kernel, W10Kernel,
                      WendlandQuinticSplineKernel)
from .nnps import (FixedDestNbrParticleLocator, NbrParticleLocatorBase,  # noqa: F401
                   NeighborLocatorType, NNPSManager, VarHNbrParticleLocator,
                   brute_force_nnps)
from .particle_array import ParticleArray  # noqa: F401
from .particle_types import ParticleType  # noqa: F401
from .particles import Particles, get_particle_array  # noqa: F401
from .point import IntPoint, Point  # noqa: F401

Fluid = ParticleType.Fluid
Solid = ParticleType.Solid
