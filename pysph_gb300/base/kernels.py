"""SPH smoothing kernels (base/kernels.pyx of the reference).

The pair kernels on the GPU evaluate the cubic spline in FP32
(``csrc/sph_internal.cuh``).  The host-side ``py_function`` /
``py_gradient`` below keep the reference's FP64 point-evaluation API
(base/kernels.pyx:104-111) with the reference's arithmetic order.
"""
import math

CUBIC_SPLINE = 1
GAUSSIAN = 2
QUINTIC_SPLINE = 3
WENDLAND_QUINTIC_SPLINE = 4
HARMONIC = 5
M6_SPLINE = 6
W8 = 7
W10 = 8
REPULSIVE = 9
POLY6 = 10


def _h_dim(h, dim):
    if dim == 1:
        return 1 / h
    if dim == 2:
        return 1 / (h * h)
    return 1 / (h * h * h)


class KernelBase:
    """Base class of the kernels (base/kernels.pyx:58)."""

    def __init__(self, dim=1, constant_h=-1):
        self.dim = int(dim)
        self.constant_h = constant_h
        self.has_constant_h = False
        self.fac = self._fac(1.0)

    def _fac(self, h):
        raise NotImplementedError("KernelBase::_fac")

    def radius(self):
        raise NotImplementedError("KernelBase::radius")

    def dimension(self):
        return self.dim

    def get_type(self):
        raise NotImplementedError("KernelBase::get_type")


class CubicSplineKernel(KernelBase):
    """Cubic spline (Monaghan 1992), base/kernels.pyx:345-449."""

    def _fac(self, h):
        dim = self.dim
        if dim == 1:
            return (2. / 3.) / h
        if dim == 2:
            return 10 / (7 * math.pi) / (h * h)
        if dim == 3:
            return 1. / math.pi / (h * h * h)
        raise ValueError("dimension must be 1, 2 or 3")

    def radius(self):
        return 2.0

    def get_type(self):
        return CUBIC_SPLINE

    def py_function(self, pa, pb, h):
        rab = math.sqrt((pa.x - pb.x) * (pa.x - pb.x) + (pa.y - pb.y) * (pa.y - pb.y) +
                        (pa.z - pb.z) * (pa.z - pb.z))
        q = rab / h
        fac = _h_dim(h, self.dim) * self.fac
        if q > 2.0:
            val = 0.0
        elif q > 1.0:
            val = 0.25 * (2 - q) * (2 - q) * (2 - q)
        else:
            val = 1 - 1.5 * (q * q) * (1 - 0.5 * q)
        return val * fac

    def py_gradient(self, pa, pb, h, grad):
        rab = math.sqrt((pa.x - pb.x) * (pa.x - pb.x) + (pa.y - pb.y) * (pa.y - pb.y) +
                        (pa.z - pb.z) * (pa.z - pb.z))
        q = rab / h
        val = 0.0
        fac = _h_dim(h, self.dim) * self.fac
        rx, ry, rz = pa.x - pb.x, pa.y - pb.y, pa.z - pb.z
        if q > 2.0:
            pass
        elif q >= 1.0:
            val = -0.75 * (2 - q) * (2 - q) / (h * rab)
        elif q > 1e-14:
            val = 3.0 * (0.75 * q - 1) / (h * h)
        grad.set(rx * (val * fac), ry * (val * fac), rz * (val * fac))


class DummyKernel(KernelBase):
    """Kernel of constant value 1 (base/kernels.pyx:328-342)."""

    def _fac(self, h):
        return 1.0

    def radius(self):
        return 2.0

    def get_type(self):
        return 0

    def py_function(self, pa, pb, h):
        return 1.0

    def py_gradient(self, pa, pb, h, grad):
        grad.set(0.0, 0.0, 0.0)


def _unsupported(name):
    class _K(KernelBase):
        def __init__(self, *a, **k):
            raise NotImplementedError(
                "%s is not part of the GPU hot path (only CubicSplineKernel)" % name)
    _K.__name__ = name
    return _K


QuinticSplineKernel = _unsupported("QuinticSplineKernel")
WendlandQuinticSplineKernel = _unsupported("WendlandQuinticSplineKernel")
GaussianKernel = _unsupported("GaussianKernel")
HarmonicKernel = _unsupported("HarmonicKernel")
M6SplineKernel = _unsupported("M6SplineKernel")
W8Kernel = _unsupported("W8Kernel")
W10Kernel = _unsupported("W10Kernel")
Poly6Kernel = _unsupported("Poly6Kernel")
