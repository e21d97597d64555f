"""SPHCalc: evaluate SPH functions of one destination over its sources.

Reference: sph/sph_calc.pyx:42-276.  ``check_internals`` raises the same
``ValueError``\\s (:132-183); ``sph`` zeroes the named outputs and sums every
source's contribution (:223-276) -- on the GPU, in one launch over all
sources.  Functions outside the hot path raise ``NotImplementedError``.
"""
import logging

import torch

from ..base.kernels import CUBIC_SPLINE, CubicSplineKernel, DummyKernel
from . import gpu

logger = logging.getLogger()

PAIR_KINDS = ("rho", "pgrad", "avisc", "xsph", "bforce", "momentum", "drho", "pilotrho", "vdiv")
RATE_KINDS = ("pgrad", "avisc", "xsph", "bforce", "momentum", "drho")


def _kind_of(func):
    kind = getattr(type(func), "gpu_kind", None)
    if kind is None:
        raise NotImplementedError("%s has no GPU implementation" % type(func).__name__)
    return kind


def _term(func, kind):
    t = {"src": func.source, "kinds": {kind}}
    if kind in ("avisc", "momentum"):
        t.update(alpha=func.alpha, beta=func.beta, eta=func.eta)
    elif kind == "xsph":
        t.update(eps=func.eps)
    elif kind == "bforce":
        t.update(delp=func.delp)
    return t


def _check_kernel(kernel, kind):
    if kind in PAIR_KINDS and kernel.get_type() != CUBIC_SPLINE:
        raise NotImplementedError("only CubicSplineKernel is implemented on the GPU")


def run_functions(particles_cm, dest, funcs, kernel, outs, accumulate=False):
    """Evaluate ``funcs`` (one per source, all one class) into ``outs``.

    ``outs`` are FP64 device tensors (or None).  With ``accumulate`` the
    results are added to ``outs`` (SPHFunction.eval), otherwise stored
    (SPHCalc.sph, which zeroes its outputs first)."""
    cm = particles_cm
    kind = _kind_of(funcs[0])
    _check_kernel(kernel, kind)
    n = dest.get_number_of_particles()
    nout = funcs[0].num_outputs
    outs = list(outs[:nout]) + [None] * (3 - min(3, nout))
    targets = outs
    if accumulate and kind in ("rho", "pilotrho", "tait", "gravity", "step"):
        targets = [None if o is None else torch.empty_like(o) for o in outs]
    if kind == "rho":
        gpu.density(cm, dest, [f.source for f in funcs], kernel.dim, targets[0])
    elif kind == "pilotrho":
        gpu.density(cm, dest, [f.source for f in funcs], kernel.dim, targets[0],
                    h0=funcs[0].h0)
    elif kind in ("adke_h", "adke_q"):
        # the reference's eval assigns the LocalReal entries; SPHCalc.sph has
        # zeroed the outputs first
        f = funcs[0]
        if targets[0] is None:
            raise ValueError("%s needs one output" % type(f).__name__)
        if not accumulate:
            targets[0].zero_()
        if kind == "adke_h":
            gpu.adke_smoothing(cm, dest, f.h0, f.k, f.eps, targets[0])
            dest.set_dirty(True)    # new neighbours are needed (adke_funcs.pyx:145-147)
        else:
            gpu.adke_conduction(cm, dest, f.g1, f.g2, targets[0])
    elif kind == "tait":
        f = funcs[0]
        if targets[0] is None or targets[1] is None:
            raise ValueError("TaitEquation needs two outputs")
        gpu.tait(cm, dest, f.co, f.ro, f.gamma, targets[0], targets[1])
    elif kind == "gravity":
        f = funcs[0]
        gpu.const_rates(cm, dest, 0, [o for o in targets[:nout]], (f.gx, f.gy, f.gz))
    elif kind == "step":
        gpu.const_rates(cm, dest, 1, [o for o in targets[:nout]])
    else:
        terms = [_term(f, kind) for f in funcs]
        if kind == "xsph":
            gpu.rates(cm, dest, terms, kernel.dim, pos=targets, accumulate=accumulate)
        elif kind in ("drho", "vdiv"):
            gpu.rates(cm, dest, terms, kernel.dim, drho=targets[0], accumulate=accumulate)
            if not accumulate:
                for o in targets[1:nout]:
                    if o is not None:
                        o.zero_()
        else:
            gpu.rates(cm, dest, terms, kernel.dim, acc=targets, accumulate=accumulate)
    if targets is not outs:
        lines = [(o, None, o, t, None, 1.0, 1) for o, t in zip(outs, targets) if o is not None]
        gpu.axpy(cm, n, lines)


class SPHCalc:
    """sph/sph_calc.pyx:42-276."""

    def __init__(self, particles, sources, dest, kernel, funcs, updates, integrates=False,
                 dnum=0, nbr_info=True, id="", kernel_gradient_correction=False,
                 kernel_correction=-1, dim=1, snum=""):
        self.nbr_info = nbr_info
        self.particles = particles
        self.sources = list(sources)
        self.nsrcs = len(self.sources)
        self.dest = dest
        self.nbr_locators = []
        self.nnps_manager = particles.nnps_manager
        self.funcs = list(funcs)
        self.kernel = kernel
        self.integrates = integrates
        self.updates = list(updates)
        self.nupdates = len(self.updates)
        self.kernel_correction = kernel_correction
        if kernel_correction != -1:
            raise NotImplementedError("kernel correction is not part of the GPU hot path")
        self.dnum = dnum
        self.id = id
        self.dim = dim
        self.snum = snum
        self.correction_manager = None
        self.tag = ""
        self.src_reads = []
        self.dst_reads = []
        self.initial_props = []
        self.dst_writes = {}
        self.check_internals()
        self.setup_internals()

    def check_internals(self):
        """sph_calc.pyx:132-183."""
        if (len(self.sources) == 0 or self.nnps_manager is None or self.dest is None or
                self.kernel is None or len(self.funcs) == 0):
            logger.debug("invalid input to setup_internals")
            return
        if len(self.funcs) != len(self.sources):
            raise ValueError("One sph function is needed per source")
        funcs = self.funcs
        for i in range(len(funcs) - 1):
            if type(funcs[i]) != type(funcs[i + 1]):
                raise ValueError("All sph_funcs should be of same type")
            if funcs[i].tag != funcs[i + 1].tag:
                raise ValueError("All functions should have the same tag")
        for i in range(len(funcs)):
            if funcs[i].source is not self.sources[i]:
                raise ValueError("SPHFunction.source not same as SPHCalc.sources[%d]" % i)
            if funcs[i].num_outputs != len(self.updates):
                raise ValueError("Number of updates not same as num_outputs; required %d, "
                                 "got %d %s for func %s" % (funcs[i].num_outputs,
                                                            len(self.updates), self.updates,
                                                            funcs[i]))

    def setup_internals(self):
        self.nbr_locators = []
        self.tag = self.funcs[0].tag
        for i in range(self.nsrcs):
            src = self.sources[i]
            func = self.funcs[i]
            func.kernel = self.kernel
            loc = self.nnps_manager.get_neighbor_particle_locator(src, self.dest,
                                                                  self.kernel.radius())
            func.nbr_locator = loc
            self.nbr_locators.append(loc)
        func = self.funcs[0]
        self.src_reads = func.src_reads
        self.dst_reads = func.dst_reads

    def sph(self, output_array1=None, output_array2=None, output_array3=None,
            exclude_self=False):
        """Zero the named outputs and evaluate every function into them."""
        names = [output_array1, output_array2, output_array3]
        outs = [self.dest.get_device(n) if n is not None else None for n in names]
        self.sph_array(outs, names, exclude_self)
        if self.dest.is_dirty:
            self.particles.update()

    def sph_array(self, outs, names=(None, None, None), exclude_self=False):
        cm = self.particles.cell_manager
        run_functions(cm, self.dest, self.funcs, self.kernel, outs, accumulate=False)
        kind = _kind_of(self.funcs[0])
        own_rho = (kind == "rho" and names[0] == "rho")
        gpu.note_written(cm, self.dest, [n for n in names if n], consistent=own_rho)


def eval_function(func, kernel, outputs):
    """``SPHFunction.eval`` on the GPU: add the result to ``outputs``."""
    dest = func.dest
    particles_cm = None
    loc = getattr(func, "nbr_locator", None)
    if loc is not None and loc.cell_manager is not None:
        particles_cm = loc.cell_manager
    if particles_cm is None:
        from ..base.cell import CellManager
        arrays = [dest] if func.source is dest else [func.source, dest]
        particles_cm = CellManager(arrays_to_bin=arrays, initialize=False)
        particles_cm._rebuild_array_indices()
        particles_cm.compute_cell_size(0, 0)
        particles_cm.initialized = True
    outs = []
    names = []
    for o in outputs:
        if o is None:
            outs.append(None)
            names.append(None)
        elif isinstance(o, str):
            outs.append(dest.get_device(o))
            names.append(o)
        else:
            outs.append(o.tensor)
            names.append(o.name)
    run_functions(particles_cm, dest, [func], kernel or func.kernel or CubicSplineKernel(dim=2),
                  outs, accumulate=True)
    gpu.note_written(particles_cm, dest, [n for n in names if n])


__all__ = ["SPHCalc", "DummyKernel"]
