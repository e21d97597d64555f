"""Solver: an ordered set of operations stepped by an integrator.

Reference: solver/solver.py:26-574 (operation bookkeeping, integrator setup,
the time loop and ``.npz`` output).
"""
import logging
import os

import numpy as np

from ..base.kernels import CubicSplineKernel, DummyKernel
from ..base.particle_types import ParticleType
from ..sph import sph_func as sph
from .integrator import EulerIntegrator
from .sph_equation import SPHIntegration

logger = logging.getLogger()

Fluids = ParticleType.Fluid


class Solver:
    def __init__(self, dim, integrator_type):
        self.particles = None
        self.integrator_type = integrator_type
        self.dim = dim
        self.default_kernel = CubicSplineKernel(dim=dim)
        self.initialize()
        self.setup_solver()
        self.with_cl = False

    def initialize(self):
        self.particles = None
        self.operation_dict = {}
        self.order = []
        self.t = 0
        self.count = 0
        self.execute_commands = None
        self.pre_step_functions = []
        self.post_step_functions = []
        self.pfreq = 100
        self.kernel_correction = -1
        self.pid = None
        self.eps = -1
        self.position_stepping_operations = {}
        self.print_properties = ["x", "u", "m", "h", "p", "rho"]
        if self.dim > 1:
            self.print_properties.extend(["y", "v"])
        if self.dim > 2:
            self.print_properties.extend(["z", "w"])
        self.fname = "solution"
        self.output_directory = "."
        self.detailed_output = False

    def switch_integrator(self, integrator_type):
        if self.particles is None:
            raise RuntimeError("There are no particles!")
        self.integrator_type = integrator_type
        self.setup_integrator(self.particles)

    def add_operation_step(self, types, xsph=False, eps=0.5):
        updates = ["x", "y", "z"][: self.dim]
        kernel = DummyKernel(dim=self.dim)
        self.add_operation(SPHIntegration(sph.PositionStepping.withargs(dim=self.dim),
                                          on_types=types, updates=updates, id="step",
                                          kernel=kernel))

    def add_operation_xsph(self, eps, hks=False):
        assert eps > 0, "Invalid value for XSPH epsilon: %f" % eps
        self.eps = eps
        assert "step" in self.operation_dict, "position stepping function does not exist!"
        types = self.operation_dict["step"].on_types
        updates = self.operation_dict["step"].updates
        self.add_operation(SPHIntegration(
            sph.XSPHCorrection.withargs(eps=eps, hks=hks, dim=self.dim), from_types=types,
            on_types=types, updates=updates, id="xsph", kernel=self.default_kernel))

    def add_operation(self, operation, before=False, id=None):
        assert operation.id not in self.order, "Operation %s exists!" % operation.id
        assert operation.id not in self.operation_dict
        self.operation_dict[operation.id] = operation
        if id:
            msg = "The specified operation doesnt exist"
            assert id in self.operation_dict, msg + " in the calcs dict!"
            assert id in self.order, msg + " in the order list!"
            if before:
                self.order.insert(self.order.index(id), operation.id)
            else:
                self.order.insert(self.order.index(id) + 1, operation.id)
        else:
            self.order.append(operation.id)

    def replace_operation(self, id, operation):
        msg = "The specified operation doesnt exist"
        assert id in self.operation_dict, msg + " in the op dict!"
        assert id in self.order, msg + " in the order list!"
        self.operation_dict.pop(id)
        self.operation_dict[operation.id] = operation
        idx = self.order.index(id)
        self.order.insert(idx, operation.id)
        self.order.remove(id)

    def remove_operation(self, id_or_operation):
        id = id_or_operation if isinstance(id_or_operation, str) else id_or_operation.id
        assert id in self.operation_dict, "id doesnt exist!"
        assert id in self.order, "id doesnt exist!"
        self.order.remove(id)
        self.operation_dict.pop(id)

    def set_order(self, order):
        for equation_id in order:
            msg = "%s in order list does not exist!" % equation_id
            assert equation_id in self.order, msg
            assert equation_id in self.operation_dict, msg
        self.order = order

    def setup_position_step(self):
        pass

    def setup_integrator(self, particles=None):
        """solver.py:320-366."""
        if particles:
            self.particles = particles
            self.particles.kernel = self.default_kernel
            self.integrator = self.integrator_type(particles, calcs=[])
            for equation_id in self.order:
                operation = self.operation_dict[equation_id]
                if operation.kernel is None:
                    operation.kernel = self.default_kernel
                self.integrator.calcs.extend(operation.get_calcs(particles, operation.kernel))
            self.integrator.setup_integrator()

    def set_final_time(self, tf):
        self.tf = tf

    def set_time_step(self, dt):
        self.dt = dt

    def set_print_freq(self, n):
        self.pfreq = n

    def set_output_fname(self, fname):
        self.fname = fname

    def set_output_printing_level(self, detailed_output):
        self.detailed_output = detailed_output

    def add_print_properties(self, props):
        for prop in props:
            if prop not in self.print_properties:
                self.print_properties.append(prop)

    def set_output_directory(self, path):
        self.output_directory = path

    def set_kernel_correction(self, kernel_correction):
        if kernel_correction != -1:
            raise NotImplementedError("kernel correction is not part of the GPU hot path")
        self.kernel_correction = kernel_correction

    def set_cl(self, with_cl=False):
        if with_cl:
            raise NotImplementedError("the OpenCL path is replaced by the CUDA path")

    def set_command_handler(self, callable, command_interval=1):
        self.execute_commands = callable
        self.command_interval = command_interval

    def solve(self, show_progress=False):
        """solver.py:457-508."""
        self.count = 0
        while self.t < self.tf:
            self.t += self.dt
            self.count += 1
            self.particles.update()
            for func in self.pre_step_functions:
                func.eval(self, self.count)
            self.integrator.integrate(self.dt)
            for func in self.post_step_functions:
                func.eval(self, self.count)
            if self.count % self.pfreq == 0:
                self.dump_output(*self.print_properties)
            if self.execute_commands is not None and self.count % self.command_interval == 0:
                self.execute_commands(self)

    def dump_output(self, *print_properties):
        """``.npz`` per array per output time (solver.py:510-538)."""
        fname = self.fname + "_"
        cell_size = self.particles.cell_manager.cell_size
        for pa in self.particles.arrays:
            name = pa.name
            _fname = os.path.join(self.output_directory, fname + name + "_" + str(self.t) + ".npz")
            if self.detailed_output:
                props = {k: pa.get(k, only_real_particles=False) for k in pa.properties}
                np.savez(_fname, dt=self.dt, **props)
            else:
                props = {prop: pa.get(prop) for prop in print_properties}
                np.savez(_fname, dt=self.dt, cell_size=cell_size, np=pa.num_real_particles,
                         **props)

    def setup_solver(self):
        pass


__all__ = ["Solver", "EulerIntegrator"]
