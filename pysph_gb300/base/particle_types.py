"""Particle array types (base/particle_types.py of the reference)."""


class ParticleType:
    """Enumeration of particle array types."""

    Fluid = 0
    Solid = 1
    DummyFluid = 2
    Probe = 3

    def __init__(self):
        raise SystemError("Do not instantiate the ParticleType class")
