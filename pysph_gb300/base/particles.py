"""Particles: the arrays of a simulation plus their neighbour structure.

Reference: base/particles.py:23-357.
"""
import numpy as np

from .cell import CellManager
from .nnps import NeighborLocatorType, NNPSManager
from .particle_array import ParticleArray
from .particle_types import ParticleType

Fluid = ParticleType.Fluid
Solid = ParticleType.Solid
Probe = ParticleType.Probe
SPHNeighborLocator = NeighborLocatorType.SPHNeighborLocator


class Particles:
    """A collection of particle arrays with one GPU cell structure."""

    def __init__(self, arrays=None, in_parallel=False, variable_h=False, load_balancing=True,
                 update_particles=True, locator_type=SPHNeighborLocator, periodic_domain=None,
                 min_cell_size=-1):
        arrays = list(arrays or [])
        assert len(arrays) > 0, "Particles must be given some arrays!"
        if in_parallel:
            raise NotImplementedError("MPI domain decomposition is not part of this build")
        prec = arrays[0].cl_precision
        for arr in arrays[1:]:
            assert arr.cl_precision == prec, "All arrays must have the same cl_precision"
        self.variable_h = variable_h
        self.in_parallel = False
        self.load_balancing = load_balancing
        self.locator_type = locator_type
        self.arrays = arrays
        self.kernel = None
        self.cell_manager = CellManager(arrays_to_bin=arrays, min_cell_size=min_cell_size,
                                        periodic_domain=periodic_domain, initialize=False)
        self.cell_manager._rebuild_array_indices()
        self.cell_manager.compute_cell_size(min_cell_size, 0)
        self.cell_manager.initialized = True
        self.nnps_manager = NNPSManager(cell_manager=self.cell_manager, variable_h=variable_h,
                                        locator_type=locator_type)
        self.correction_manager = None
        self.misc_prop_update_functions = []
        if update_particles:
            self.update()

    def update(self, cache_neighbors=False):
        """Rebuild the neighbour structure of moved arrays (particles.py:159-200)."""
        err = self.nnps_manager.py_update()
        assert err != -1, "NNPSManager update failed! "
        self.evaluate_misc_properties()

    def evaluate_misc_properties(self):
        for func in self.misc_prop_update_functions:
            func.eval()

    def add_misc_function(self, func, operation, kernel):
        calcs = operation.get_calcs(self, kernel)
        self.misc_prop_update_functions.append(func(calcs))

    def get_named_particle_array(self, name):
        for array in self.arrays:
            if array.name == name:
                return array
        print("Array %s does not exist!" % name)
        return None

    def update_remote_particle_properties(self, props=None):
        return None

    def barrier(self):
        return None

    @classmethod
    def get_neighbor_particle_locator(cls, src, dst, locator_type=SPHNeighborLocator,
                                      variable_h=False, radius_scale=2.0):
        arrays = [src] if src is dst else [src, dst]
        cm = CellManager(arrays_to_bin=arrays, initialize=False)
        cm._rebuild_array_indices()
        cm.compute_cell_size(0, 0)
        cm.initialized = True
        nm = NNPSManager(cm, locator_type=locator_type, variable_h=variable_h)
        return nm.get_neighbor_particle_locator(src, dst, radius_scale)

    def get_cl_precision(self):
        return self.arrays[0].cl_precision

    # -- extension: FP64 invariants on the GPU ----------------------------------
    def invariants(self, array=None):
        """FP64 sums over LocalReal particles of one array (default: all):
        ``dict(mass, momentum(3), kinetic_energy, count)``."""
        import ctypes

        from .. import native
        from .cell import array_view
        arrays = self.arrays if array is None else [array]
        tot = np.zeros(6)
        ctx = self.cell_manager.context()
        for pa in arrays:
            out = (ctypes.c_double * 6)()
            v = array_view(pa)
            native.check(native.lib().sph_invariants(ctx, ctypes.byref(v), out), "invariants")
            tot += np.array(out[:])
        return {"mass": tot[0], "momentum": tot[1:4], "kinetic_energy": tot[4],
                "count": int(tot[5])}


def get_particle_array(cl_precision="double", **props):
    """particles.py:282-356: build a ParticleArray with the default properties."""
    prop_dict = {}
    name = ""
    particle_type = Fluid
    default_props = {"x": 0.0, "y": 0.0, "z": 0.0, "u": 0.0, "v": 0.0, "w": 0.0, "m": 1.0,
                     "h": 1.0, "p": 0.0, "e": 0.0, "rho": 1.0, "cs": 0.0}
    np_ = 0
    for prop in props:
        if prop in ("name", "type"):
            continue
        np_ = len(props[prop])
        if prop == "idx":
            prop_dict[prop] = {"data": np.asarray(props[prop]), "type": "long"}
        else:
            prop_dict[prop] = {"data": np.asarray(props[prop]), "type": "double"}
    for prop, default in default_props.items():
        if prop not in props:
            prop_dict[prop] = {"name": prop, "type": "double", "default": default}
    if "idx" not in prop_dict and np_ != 0:
        prop_dict["idx"] = {"name": "idx", "data": np.arange(np_), "type": "long"}
    if "name" in props:
        name = props["name"]
    if "type" in props:
        particle_type = props["type"]
        assert particle_type in (Fluid, Solid, Probe), "Type not understood!"
    return ParticleArray(name=name, particle_type=particle_type, cl_precision=cl_precision,
                         **prop_dict)
