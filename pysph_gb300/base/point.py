"""Point types (base/point.pyx of the reference), host side only."""
import math

import numpy as np


class Point:
    """A point in 3D (``base/point.pyx`` ``Point``)."""

    __slots__ = ("x", "y", "z")

    def __init__(self, x=0.0, y=0.0, z=0.0):
        self.x, self.y, self.z = float(x), float(y), float(z)

    def set(self, x, y, z):
        self.x, self.y, self.z = float(x), float(y), float(z)

    def asarray(self):
        return np.array([self.x, self.y, self.z])

    def norm(self):
        """Squared length (``cPoint_norm``, base/point.pxd:26-27)."""
        return self.x * self.x + self.y * self.y + self.z * self.z

    def length(self):
        return math.sqrt(self.norm())

    def dot(self, p):
        return self.x * p.x + self.y * p.y + self.z * p.z

    def cross(self, p):
        return Point(self.y * p.z - self.z * p.y, self.z * p.x - self.x * p.z,
                     self.x * p.y - self.y * p.x)

    def distance(self, p):
        return math.sqrt((self.x - p.x) ** 2 + (self.y - p.y) ** 2 + (self.z - p.z) ** 2)

    def __add__(self, p):
        return Point(self.x + p.x, self.y + p.y, self.z + p.z)

    def __sub__(self, p):
        return Point(self.x - p.x, self.y - p.y, self.z - p.z)

    def __mul__(self, k):
        return Point(self.x * k, self.y * k, self.z * k)

    def __eq__(self, p):
        return isinstance(p, Point) and (self.x, self.y, self.z) == (p.x, p.y, p.z)

    def __repr__(self):
        return "Point(%g, %g, %g)" % (self.x, self.y, self.z)


class IntPoint:
    __slots__ = ("x", "y", "z")

    def __init__(self, x=0, y=0, z=0):
        self.x, self.y, self.z = int(x), int(y), int(z)

    def __hash__(self):
        return hash((self.x, self.y, self.z))

    def __eq__(self, p):
        return isinstance(p, IntPoint) and (self.x, self.y, self.z) == (p.x, p.y, p.z)

    def copy(self):
        return IntPoint(self.x, self.y, self.z)

    def __repr__(self):
        return "IntPoint(%d, %d, %d)" % (self.x, self.y, self.z)
