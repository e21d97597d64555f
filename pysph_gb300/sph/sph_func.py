"""SPH function classes with the reference's constructors and attributes.

Reference: sph/sph_func.pyx (``Function`` :25-77, ``SPHFunction`` :82,
``SPHFunctionParticle`` :338, ``CSPHFunctionParticle`` :457) and the
function modules under sph/funcs/.  The classes here carry the parameters
and the ``num_outputs`` / ``tag`` / ``id`` bookkeeping the calcs and the
integrator rely on; the arithmetic runs in the GPU kernels selected by each
class's ``gpu_kind``.
"""
from ..base.particle_array import ParticleArray


class Function:
    """An SPH function class with bound constructor arguments (:25-77)."""

    def __init__(self, sph_func, *args, **kwargs):
        self.sph_func = sph_func
        self.args = args
        self.kwargs = kwargs

    def get_func_class(self):
        return self.sph_func

    def get_func(self, source, dest):
        return self.sph_func(source, dest, *self.args, **self.kwargs)


class SPHFunction:
    """An operation on a destination particle array (:82-336)."""

    gpu_kind = None   # name of the GPU evaluation this class maps to

    def __init__(self, source, dest=None, setup_arrays=True, *args, **kwargs):
        if not isinstance(source, ParticleArray):
            raise TypeError("source must be a ParticleArray")
        self.name = ""
        self.id = ""
        self.tag = ""
        self.source = source
        self.dest = source
        for p in ("x", "y", "z", "u", "v", "w", "m", "rho", "h", "p", "e", "cs"):
            setattr(self, p, p)
        self.num_outputs = 3
        self.src_reads = []
        self.dst_reads = []
        self.kernel = None
        self.nbr_locator = None
        self.exclude_self = False
        self.hks = False
        self.set_src_dst_reads()

    @classmethod
    def withargs(cls, *args, **kwargs):
        return Function(cls, *args, **kwargs)

    @classmethod
    def get_func(cls, source, dest):
        return Function(cls).get_func(source, dest)

    @classmethod
    def get_func_class(cls):
        return cls

    def set_src_dst_reads(self):
        pass

    def setup_arrays(self):
        pass

    def setup_iter_data(self):
        pass

    def eval(self, kernel, output1=None, output2=None, output3=None):
        """Add this function's result to the outputs (sph_func.pyx:199-234).

        ``outputN`` are the carrays of ``dest.get_carray(name)`` (or property
        names).  Evaluated on the GPU like a one-function ``SPHCalc``."""
        from .sph_calc import eval_function
        eval_function(self, kernel, [output1, output2, output3])


class SPHFunctionParticle(SPHFunction):
    """An interaction between a source and a destination array (:338-455)."""

    def __init__(self, source, dest, setup_arrays=True, hks=False, exclude_self=False,
                 nbr_locator=None, *args, **kwargs):
        SPHFunction.__init__(self, source, setup_arrays=False)
        self.dest = dest
        self.exclude_self = exclude_self
        self.hks = hks
        self.nbr_locator = nbr_locator
        self.bonnet_and_lok_correction = False
        self.rkpm_first_order_correction = False
        if hks:
            raise NotImplementedError("hks=True kernel symmetrisation is not part of the GPU hot path")
        if exclude_self:
            raise NotImplementedError(
                "exclude_self=True: the reference's eval_single reads an undefined "
                "attribute in this case (sph_func.pyx:388); only the default works")


class CSPHFunctionParticle(SPHFunctionParticle):
    """Corrected-SPH base (:457-493); without kernel correction the
    denominator stays zero and the sum is returned unchanged."""


# ---------------------------------------------------------------------------
# hot-path functions
# ---------------------------------------------------------------------------

class SPHRho(CSPHFunctionParticle):
    """Summation density, sph/funcs/density_funcs.pyx:15-84."""

    gpu_kind = "rho"

    def __init__(self, source, dest, setup_arrays=True, **kwargs):
        SPHFunctionParticle.__init__(self, source, dest, setup_arrays=True, **kwargs)
        self.id = "sphrho"
        self.tag = "density"
        self.num_outputs = 1

    def set_src_dst_reads(self):
        self.src_reads = ["x", "y", "z", "h", "m"]
        self.dst_reads = ["x", "y", "z", "h", "tag"]


class TaitEquation(SPHFunction):
    """Tait equation of state, sph/funcs/eos_funcs.pyx:58-117."""

    gpu_kind = "tait"

    def __init__(self, source, dest, setup_arrays=True, co=1.0, ro=1000.0, gamma=7.0, **kwargs):
        SPHFunction.__init__(self, source, dest, setup_arrays)
        self.co = float(co)
        self.ro = float(ro)
        self.gamma = float(gamma)
        self.B = co * co * ro / gamma
        self.id = "tait"
        self.tag = "state"
        self.num_outputs = 2

    def set_src_dst_reads(self):
        self.src_reads = []
        self.dst_reads = ["rho"]


class SPHPressureGradient(SPHFunctionParticle):
    """sph/funcs/pressure_funcs.pyx:12-98."""

    gpu_kind = "pgrad"

    def __init__(self, source, dest, setup_arrays=True, dim=3, **kwargs):
        SPHFunctionParticle.__init__(self, source, dest, setup_arrays, **kwargs)
        self.id = "pgrad"
        self.tag = "velocity"
        self.num_outputs = int(dim)

    def set_src_dst_reads(self):
        self.src_reads = ["x", "y", "z", "h", "m", "rho", "p"]
        self.dst_reads = ["x", "y", "z", "h", "rho", "p", "tag"]


class MonaghanArtificialVsicosity(SPHFunctionParticle):
    """sph/funcs/viscosity_funcs.pyx:10-124.

    The reference's constructor accepts ``eta`` but never stores it
    (:21-34), so ``self.eta`` stays 0.0 and the denominator of mu is
    ``|r_ab|^2`` alone; reproduced here."""

    gpu_kind = "avisc"

    def __init__(self, source, dest, setup_arrays=True, alpha=1, beta=1, gamma=1.4, eta=0.1,
                 **kwargs):
        SPHFunctionParticle.__init__(self, source, dest, setup_arrays, **kwargs)
        self.alpha = float(alpha)
        self.beta = float(beta)
        self.gamma = float(gamma)
        self.eta = 0.0
        self.id = "momavisc"
        self.tag = "velocity"

    def set_src_dst_reads(self):
        self.src_reads = ["x", "y", "z", "h", "m", "rho", "u", "v", "w", "cs"]
        self.dst_reads = ["x", "y", "z", "h", "p", "u", "v", "w", "cs", "rho", "tag"]


class MomentumEquation(SPHFunctionParticle):
    """sph/funcs/pressure_funcs.pyx:106-252: the pressure gradient and the
    Monaghan viscosity in one pair term.  Unlike MonaghanArtificialVsicosity
    it stores ``eta``, so mu's denominator is |r_ab|^2 + eta^2 hab^2."""

    gpu_kind = "momentum"

    def __init__(self, source, dest, setup_arrays=True, alpha=1, beta=1, gamma=1.4, eta=0.1,
                 dim=3, **kwargs):
        SPHFunctionParticle.__init__(self, source, dest, setup_arrays, **kwargs)
        self.alpha = float(alpha)
        self.beta = float(beta)
        self.gamma = float(gamma)
        self.eta = float(eta)
        self.id = "momentumequation"
        self.tag = "velocity"
        self.num_outputs = int(dim)

    def set_src_dst_reads(self):
        self.src_reads = ["x", "y", "z", "h", "m", "rho", "p", "u", "v", "w", "cs"]
        self.dst_reads = ["x", "y", "z", "h", "rho", "p", "u", "v", "w", "cs", "tag"]


class SPHDensityRate(SPHFunctionParticle):
    """sph/funcs/density_funcs.pyx:89-158: drho_a/dt = sum_b m_b v_ab . grad W(hab)."""

    gpu_kind = "drho"

    def __init__(self, source, dest, setup_arrays=True, **kwargs):
        SPHFunctionParticle.__init__(self, source, dest, True, **kwargs)
        self.id = "densityrate"
        self.tag = "density"
        self.num_outputs = 1

    def set_src_dst_reads(self):
        self.src_reads = ["x", "y", "z", "h", "m", "u", "v", "w"]
        self.dst_reads = ["x", "y", "z", "h", "tag", "u", "v", "w"]


class XSPHCorrection(CSPHFunctionParticle):
    """sph/funcs/xsph_funcs.pyx:8-88."""

    gpu_kind = "xsph"

    def __init__(self, source, dest, setup_arrays=True, eps=0.5, dim=3, **kwargs):
        CSPHFunctionParticle.__init__(self, source, dest, setup_arrays, **kwargs)
        self.eps = float(eps)
        self.id = "xsph"
        self.tag = "position"
        self.num_outputs = int(dim)

    def set_src_dst_reads(self):
        self.src_reads = ["x", "y", "z", "h", "m", "rho", "u", "v", "w"]
        self.dst_reads = ["x", "y", "z", "h", "rho", "u", "v", "w"]


class PositionStepping(SPHFunction):
    """sph/funcs/position_funcs.pyx:10-60 (k = velocity)."""

    gpu_kind = "step"

    def __init__(self, source, dest, setup_arrays=True, dim=3):
        SPHFunction.__init__(self, source, dest, setup_arrays)
        self.id = "positionstepper"
        self.tag = "position"
        self.num_outputs = int(dim)

    def set_src_dst_reads(self):
        self.src_reads = []
        self.dst_reads = ["u", "v", "w"][: self.num_outputs]


class MonaghanBoundaryForce(SPHFunctionParticle):
    """sph/funcs/boundary_funcs.pyx:10-110 (needs tx..nz on the source)."""

    gpu_kind = "bforce"

    def __init__(self, source, dest, setup_arrays=False, delp=1.0, **kwargs):
        SPHFunctionParticle.__init__(self, source, dest, setup_arrays=True, **kwargs)
        self.id = "monaghanbforce"
        self.tag = "velocity"
        self.delp = float(delp)
        for p in ("tx", "ty", "tz", "nx", "ny", "nz"):
            if not source.has_array(p):
                raise AttributeError("property %s not present" % p)

    def set_src_dst_reads(self):
        self.src_reads = ["x", "y", "z", "h", "m", "rho", "tx", "ty", "tz", "nx", "ny", "nz", "cs"]
        self.dst_reads = ["x", "y", "z", "h", "m", "cs", "tag"]


class GravityForce(SPHFunction):
    """sph/funcs/external_force.pyx:14-63."""

    gpu_kind = "gravity"

    def __init__(self, source, dest, setup_arrays=True, gx=0.0, gy=0.0, gz=0.0, hks=False):
        SPHFunction.__init__(self, source, dest, setup_arrays)
        self.id = "gravityforce"
        self.tag = "velocity"
        self.gx = float(gx)
        self.gy = float(gy)
        self.gz = float(gz)


# ---------------------------------------------------------------------------
# ADKE: Sigalotti's adaptive kernel estimation (sph/funcs/adke_funcs.pyx)
# ---------------------------------------------------------------------------

class ADKEPilotRho(CSPHFunctionParticle):
    """Pilot density sum m_b W(x_a - x_b, h0) at a fixed h0, over the
    neighbours of the destination's own radius (adke_funcs.pyx:15-73)."""

    gpu_kind = "pilotrho"

    def __init__(self, source, dest, setup_arrays=True, h0=1.0, **kwargs):
        SPHFunctionParticle.__init__(self, source, dest, True, **kwargs)
        self.h0 = float(h0)
        if not self.h0 > 0.0:
            raise ValueError("ADKEPilotRho: h0 must be positive")
        self.id = "pilotrho"
        self.tag = "pilotrho"
        self.num_outputs = 1

    def set_src_dst_reads(self):
        self.src_reads = ["x", "y", "z", "m", "rho"]
        self.dst_reads = ["x", "y", "z", "tag"]


class ADKESmoothingUpdate(SPHFunction):
    """h_a = h0 k (g / rhop_a)^eps with log g the mean of log rhop over the
    LocalReal particles (adke_funcs.pyx:78-147); marks the array dirty, since
    new neighbours are needed."""

    gpu_kind = "adke_h"

    def __init__(self, source, dest, setup_arrays=True, k=1.0, eps=0.0, h0=1.0, **kwargs):
        SPHFunction.__init__(self, source, dest, setup_arrays)
        self.dest = dest if dest is not None else source
        self.k = float(k)
        self.eps = float(eps)
        self.h0 = float(h0)
        self.id = "adke_smoothing_update"
        self.tag = "h"
        self.num_outputs = 1

    def set_src_dst_reads(self):
        self.src_reads = []
        self.dst_reads = ["rhop"]


class SPHVelocityDivergence(SPHFunctionParticle):
    """(1/rho_a) sum m_b (v_b - v_a) . grad W(r_ab, (h_a + h_b)/2)
    (adke_funcs.pyx:152-226).  Like the reference class it keeps
    SPHFunction's three outputs (the second and third stay zero)."""

    gpu_kind = "vdiv"

    def __init__(self, source, dest, setup_arrays=True, **kwargs):
        SPHFunctionParticle.__init__(self, source, dest, True, **kwargs)
        self.id = "vdivergence"
        self.tag = "vdivergence"

    def set_src_dst_reads(self):
        self.src_reads = ["x", "y", "z", "h", "u", "v", "w", "m"]
        self.dst_reads = ["x", "y", "z", "h", "u", "v", "w", "rho", "tag"]


VelocityDivergence = SPHVelocityDivergence


class ADKEConductionCoeffUpdate(SPHFunction):
    """q_a = (g1 c_a + g2 h_a (|div_a| - div_a)) h_a over the LocalReal
    particles (adke_funcs.pyx:231-291)."""

    gpu_kind = "adke_q"

    def __init__(self, source, dest, setup_arrays=True, g1=0.0, g2=0.0, **kwargs):
        SPHFunction.__init__(self, source, dest, setup_arrays)
        self.dest = dest if dest is not None else source
        self.g1 = float(g1)
        self.g2 = float(g2)
        self.id = "adke_conduction"
        self.tag = "q"
        self.num_outputs = 1

    def set_src_dst_reads(self):
        self.src_reads = ["x", "y", "z", "h", "u", "v", "w", "m"]
        self.dst_reads = ["x", "y", "z", "h", "u", "v", "w", "rho", "cs", "tag"]


def _not_on_gpu(name, ref):
    class _F(SPHFunctionParticle):
        def __init__(self, *a, **k):
            raise NotImplementedError("%s (%s) is not part of the GPU hot path" % (name, ref))
    _F.__name__ = name
    return _F


MorrisViscosity = _not_on_gpu("MorrisViscosity", "sph/funcs/viscosity_funcs.pyx:129")
IdealGasEquation = _not_on_gpu("IdealGasEquation", "sph/funcs/eos_funcs.pyx:13")
XSPHDensityRate = _not_on_gpu("XSPHDensityRate", "sph/funcs/xsph_funcs.pyx:96")
BeckerBoundaryForce = _not_on_gpu("BeckerBoundaryForce", "sph/funcs/boundary_funcs.pyx:116")
VectorForce = _not_on_gpu("VectorForce", "sph/funcs/external_force.pyx:68")
NBodyForce = _not_on_gpu("NBodyForce", "sph/funcs/external_force.pyx")
