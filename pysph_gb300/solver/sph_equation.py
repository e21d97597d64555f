"""SPHOperation / SPHIntegration: expand an equation into calcs.

Reference: solver/sph_equation.py:10-254 (same grouping of particle arrays
into destination/source pairs, same calc ids and error behaviour).
"""
from ..base.particle_types import ParticleType
from ..sph.sph_calc import SPHCalc
from ..sph.sph_func import SPHFunctionParticle

Fluid = ParticleType.Fluid
Solid = ParticleType.Solid


class SPHOperation:
    def __init__(self, function, on_types, updates, id, kernel=None, from_types=None,
                 kernel_correction=-1, integrates=False):
        self.from_types = list(from_types or [])
        self.on_types = list(on_types)
        self.function = function
        self.updates = list(updates)
        self.id = id
        self.integrates = integrates
        self.kernel = kernel
        self.nbr_info = issubclass(function.get_func_class(), SPHFunctionParticle)
        self.kernel_correction = kernel_correction
        self.has_kernel_correction = kernel_correction != -1
        self.calc_type = SPHCalc

    def get_calc_data(self, particles):
        """sph_equation.py:101-166."""
        arrays = particles.arrays
        calc_data = {}
        for i, dst in enumerate(arrays):
            if dst.particle_type not in self.on_types:
                continue
            calc_data[i] = {"sources": [], "funcs": [], "dnum": i, "id": "", "snum": str(i)}
            if self.from_types == []:
                func = self.function.get_func(dst, dst)
                func.id = self.id
                calc_data[i]["funcs"] = [func]
                calc_data[i]["id"] = self.id + "_" + dst.name
            else:
                for j, src in enumerate(arrays):
                    if src.particle_type in self.from_types:
                        func = self.function.get_func(source=src, dest=dst)
                        func.id = self.id
                        calc_data[i]["sources"].append(src)
                        calc_data[i]["funcs"].append(func)
                        calc_data[i]["snum"] = calc_data[i]["snum"] + str(j)
                        calc_data[i]["id"] = self.id + "_" + dst.name
                if calc_data[i]["sources"] == []:
                    raise RuntimeWarning("No source found for %s operation" % self.id)
        return calc_data

    def get_calcs(self, particles, kernel):
        calcs = []
        calc_data = self.get_calc_data(particles)
        for i, dest in enumerate(particles.arrays):
            if i in calc_data:
                d = calc_data[i]
                calcs.append(self.calc_type(
                    particles=particles, sources=d["sources"], dest=dest, funcs=d["funcs"],
                    kernel=kernel, updates=self.updates, integrates=self.integrates,
                    dnum=d["dnum"], id=d["id"], dim=kernel.dim, snum=d["snum"],
                    kernel_correction=self.kernel_correction, nbr_info=self.nbr_info))
        return calcs


class SPHIntegration(SPHOperation):
    """An integrating SPHOperation (sph_equation.py:227-254)."""

    def __init__(self, function, on_types, updates, id, kernel=None, from_types=None,
                 kernel_correction=-1):
        SPHOperation.__init__(self, function, on_types, updates, id, kernel,
                              from_types=from_types, integrates=True,
                              kernel_correction=kernel_correction)
