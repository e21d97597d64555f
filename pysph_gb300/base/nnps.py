"""Neighbour queries over the GPU cell structure.

Reference: base/nnps.pyx.  ``FixedDestNbrParticleLocator`` (:385-650) kept a
``LongArray`` of neighbours per destination particle, rebuilt whenever an
array moved.  The GPU pair kernels need no such cache: they walk the sorted
cell rows directly.  The locator here serves the API: its neighbour lists
are exported from the device on first query after a rebuild (FP64 distance
test ``|x_j - x_i|^2 < (radius_scale h_i)^2`` as in :337-353, each list in
ascending index order with the particle itself then swapped with the last
entry, as the reference's cache update does, :609-616).
"""
import ctypes

import numpy as np
import torch

from .. import native
from .carray import DoubleArray, LongArray
from .point import Point


class NeighborLocatorType:
    SPHNeighborLocator = 0
    NSquareNeighborLocator = 1


def brute_force_nnps(pnt, search_radius, xa, ya, za, neighbor_indices, neighbor_distances,
                     exclude_index=-1):
    """base/nnps.pyx:78-94 (host, O(N))."""
    xa, ya, za = (np.asarray(a, np.float64) for a in (xa, ya, za))
    d = (pnt.x - xa) ** 2 + (pnt.y - ya) ** 2 + (pnt.z - za) ** 2
    r2 = search_radius * search_radius
    sel = np.nonzero((d <= r2) & (np.arange(d.size) != exclude_index))[0]
    for i in sel:
        neighbor_indices.append(int(i))
        neighbor_distances.append(float(d[i]))


def get_distance_matrix(xa, ya, za):
    x, y, z = (np.asarray(a, np.float64) for a in (xa, ya, za))
    d = (x[None, :] - x[:, None]) ** 2 + (y[None, :] - y[:, None]) ** 2 + \
        (z[None, :] - z[:, None]) ** 2
    return np.sqrt(d)


def get_adjacency_matrix(xa, ya, za, ha, radius_scale=1.0):
    dist = get_distance_matrix(xa, ya, za)
    return dist < np.asarray(ha)[:, None] * radius_scale


def get_distance_matrix_pa(parray):
    return get_distance_matrix(parray.get("x"), parray.get("y"), parray.get("z"))


def get_adjacency_matrix_pa(parray, radius_scale=1.0):
    return get_adjacency_matrix(parray.get("x"), parray.get("y"), parray.get("z"),
                                parray.get("h"), radius_scale)


class NbrParticleLocatorBase:
    def __init__(self, source, cell_manager=None):
        self.cell_manager = cell_manager
        self.source = source
        self.source_index = -1
        self.locator_type = NeighborLocatorType.SPHNeighborLocator
        if cell_manager is not None:
            self.source_index = cell_manager.array_indices.get(source.name)
            if self.source_index is None:
                raise ValueError("Source %s does not exist" % source.name)

    def set_locator_type(self, locator_type):
        self.locator_type = locator_type

    def py_get_nearest_particles_to_point(self, pnt, radius, output_array, exclude_index=-1):
        """All source particles with ``|x_j - pnt|^2 < radius^2`` (host query)."""
        xs, ys, zs = (self.source.get(c, only_real_particles=False) for c in ("x", "y", "z"))
        d2 = (xs - pnt.x) * (xs - pnt.x) + (ys - pnt.y) * (ys - pnt.y) + (zs - pnt.z) * (zs - pnt.z)
        for j in np.nonzero(d2 < radius * radius)[0]:
            if j != exclude_index:
                output_array.append(int(j))
        return 0


class FixedDestNbrParticleLocator(NbrParticleLocatorBase):
    """Neighbours of every ``dest`` particle among ``source`` particles."""

    def __init__(self, source, dest, radius_scale, cell_manager=None, h="h"):
        super().__init__(source, cell_manager)
        self.dest = dest
        self.radius_scale = radius_scale
        self.h = h
        self.dest_index = -1
        self.is_dirty = True
        self._csr = None
        self._build = -1
        if cell_manager is not None:
            self.dest_index = cell_manager.array_indices.get(dest.name)
            if self.dest_index is None:
                raise ValueError("Destination %s does not exist" % dest.name)

    def update_status(self):
        if not self.is_dirty:
            self.is_dirty = self.source.is_dirty or self.dest.is_dirty

    def py_update_status(self):
        self.update_status()

    def update(self):
        cm = self.cell_manager
        cm.ensure_current()
        if self.is_dirty or self._build != cm._build_count or self._csr is None:
            self._csr = self._export()
            self._build = cm._build_count
            self.is_dirty = False
        return 0

    def py_update(self):
        return self.update()

    def _export(self):
        cm = self.cell_manager
        L = native.lib()
        ctx = cm.context()
        n = self.dest.get_number_of_particles()
        dev = torch.device("cuda")
        counts = torch.zeros(max(n, 1), dtype=torch.int64, device=dev)
        native.check(L.sph_nnps_count(ctx, self.dest_index, self.source_index,
                                      self.radius_scale, ctypes.c_void_p(counts.data_ptr())),
                     "neighbour count")
        c = counts[:n].cpu().numpy()
        offsets = np.zeros(n + 1, np.int64)
        np.cumsum(c, out=offsets[1:])
        off_d = torch.as_tensor(offsets, device=dev)
        index = torch.zeros(max(int(offsets[-1]), 1), dtype=torch.int64, device=dev)
        native.check(L.sph_nnps_fill(ctx, self.dest_index, self.source_index, self.radius_scale,
                                     ctypes.c_void_p(off_d.data_ptr()),
                                     ctypes.c_void_p(index.data_ptr())), "neighbour fill")
        return offsets, index[: offsets[-1]].cpu().numpy()

    def neighbour_csr(self):
        """All lists at once: ``(offsets, index)`` (int64 NumPy arrays)."""
        self.update()
        return self._csr

    def py_get_nearest_particles(self, dest_p_index, exclude_self=False):
        if self.locator_type == NeighborLocatorType.NSquareNeighborLocator:
            n = self.source.get_number_of_particles()
            idx = list(range(n))
            if self.dest is self.source and exclude_self:
                idx[dest_p_index], idx[n - 1] = idx[n - 1], idx[dest_p_index]
                idx = idx[:-1]
            out = LongArray(len(idx))
            out.set_data(np.asarray(idx, np.int64))
            return out
        self.update()
        off, idx = self._csr
        lst = idx[off[dest_p_index]:off[dest_p_index + 1]]
        if self.dest is self.source and exclude_self:
            lst = lst[:-1]
        out = LongArray(lst.size)
        out.set_data(lst)
        return out


class VarHNbrParticleLocator(FixedDestNbrParticleLocator):
    """base/nnps.pyx:654-749: neighbours for per-particle smoothing lengths,
    symmetric -- j is a neighbour of i when i is within the radius of j or j
    within the radius of i.  The reference builds the union from a reversed
    locator; here the cell manager's device build applies both tests (its
    context is switched to the symmetric relation), so every pair pass and
    exported list of that manager sees the union."""

    def __init__(self, source, dest, radius_scale, cell_manager=None, h="h"):
        if cell_manager is not None:
            cell_manager.set_symmetric(True)
        FixedDestNbrParticleLocator.__init__(self, source, dest, radius_scale, cell_manager)


class NNPSManager:
    """base/nnps.pyx:754-895."""

    def __init__(self, cell_manager=None, variable_h=False,
                 locator_type=NeighborLocatorType.SPHNeighborLocator):
        self.cell_manager = cell_manager
        if variable_h and cell_manager is not None:
            cell_manager.set_symmetric(True)
        self.variable_h = variable_h
        self.locator_type = locator_type
        self.particle_locator_cache = {}
        self.polygon_cache = {}

    def get_neighbor_particle_locator(self, source, dest=None, radius_scale=1.0):
        if dest is None:
            dest = source
        key = (source.name, dest.name, float(radius_scale))
        loc = self.particle_locator_cache.get(key)
        if loc is None:
            cls = VarHNbrParticleLocator if self.variable_h else FixedDestNbrParticleLocator
            loc = cls(source, dest, radius_scale, self.cell_manager)
            loc.set_locator_type(self.locator_type)
            self.particle_locator_cache[key] = loc
        return loc

    def py_update(self):
        if self.cell_manager is not None:
            self.cell_manager.update()
        for loc in self.particle_locator_cache.values():
            loc.update_status()
        return 0

    def update(self):
        return self.py_update()
