"""Many independent simulations of one recipe, advanced together on the GPU.

The reference runs one simulation per ``Solver``.  A ``SimulationBatch``
takes N instances that share an operation recipe -- summation density of
the instance on itself (optionally followed by the Tait equation), one set of
rate terms among the instance's own particles (pressure gradient, Monaghan
artificial viscosity, XSPH), gravity, position stepping, Euler or RK2 -- and
advances all of them with one fixed sequence of launches per step, captured
in a CUDA graph (``sph_batch_*`` in ``include/pysph_gb300.h``).

Each instance keeps its own smoothing length, cell size and cell
subdivision (its own dense grid over a region around its particles), so
instances of very different resolution share the launches without sharing
cells.  The regions follow the instances: a step in which a particle leaves
its instance's region is undone on the device and repeated on regions
re-derived from the current extents (``margin``).
"""
import ctypes

import numpy as np
import torch

from . import native
from .base import transfer

PROPS = ("x", "y", "z", "u", "v", "w", "m", "h", "rho", "p", "cs")


class SimulationBatch:
    """``instances``: list of property dicts (NumPy, as for
    ``get_particle_array``).  Physics: SPHRho, Tait(co, ro, gamma), then
    the rate terms named by ``terms`` (subset of pgrad, avisc, xsph) with
    ``alpha``, ``beta``, ``eps``, optional ``gravity`` and position stepping,
    integrated with ``integrator`` ('euler' or 'rk2') at ``dt``.

    ``subdiv``: the cell subdivision (1..3), one for all instances or a
    sequence with one per instance (``tuning.autotune_batch`` chooses them);
    ``margin``: the regions are the instances' extents grown by ``margin``
    times the extent plus four reference cells on every side (0: fixed
    regions, leaving one is an error)."""

    def __init__(self, instances, dim=2, dt=1e-5, co=100.0, ro=1.0, gamma=7.0,
                 terms=("pgrad", "avisc", "xsph"), alpha=0.01, beta=0.0, eps=0.5,
                 gravity=None, step_positions=True, integrator="euler", radius_scale=2.0,
                 margin=0.25, subdiv=None, list_cap=0, use_graph=True):
        if not instances:
            raise ValueError("a batch needs at least one instance")
        if not torch.cuda.is_available():
            raise RuntimeError("pysph_gb300 needs a CUDA device (GB300, sm_103a); "
                               "there is no CPU fallback")
        self.dim = int(dim)
        self.dt = float(dt)
        self.use_graph = use_graph
        n_each = [len(p["x"]) for p in instances]
        self.offsets = np.concatenate([[0], np.cumsum(n_each)]).astype(np.int64)
        self.n = int(self.offsets[-1])
        dev = torch.device("cuda")
        defaults = {"y": 0.0, "z": 0.0, "u": 0.0, "v": 0.0, "w": 0.0, "m": 1.0, "h": 1.0,
                    "rho": 1.0, "p": 0.0, "cs": 0.0}
        host = {}
        for name in PROPS:
            parts = []
            for p, k in zip(instances, n_each):
                a = p.get(name)
                parts.append(np.full(k, defaults.get(name, 0.0)) if a is None
                             else np.asarray(a, np.float64))
            host[name] = np.concatenate(parts)
        self.arrays = {k: torch.as_tensor(v, device=dev).clone() for k, v in host.items()}
        view = native.ArrayView()
        view.n = self.n
        for f in native.VIEW_FIELDS:
            t = self.arrays.get(f)
            setattr(view, f, None if t is None else t.data_ptr())
        view.tag = None
        self._view = view

        ninst = len(instances)
        from .tuning import DEFAULT_SUBDIVISION
        if subdiv is None:
            subdiv = DEFAULT_SUBDIVISION[self.dim]
        per_inst = [int(subdiv)] * ninst if np.isscalar(subdiv) else [int(v) for v in subdiv]
        if len(per_inst) != ninst or any(v not in (1, 2, 3) for v in per_inst):
            raise ValueError("subdiv: 1, 2 or 3, or one such value per instance")
        self.subdiv = per_inst
        inst = (native.BatchInstance * ninst)()
        for k in range(ninst):
            a, b = int(self.offsets[k]), int(self.offsets[k + 1])
            h = host["h"][a:b]
            inst[k].offset = a
            inst[k].n = b - a
            inst[k].cell_size = radius_scale * float(h.max())
            inst[k].uniform_h = int(h.min() == h.max())
            inst[k].subdiv = per_inst[k]
            for d, c in enumerate(("x", "y", "z")):
                lo, hi = float(host[c][a:b].min()), float(host[c][a:b].max())
                ext = hi - lo
                pad = margin * ext + 4.0 * inst[k].cell_size if ext > 0 else 0.0
                inst[k].lo[d] = lo - pad
                inst[k].hi[d] = hi + pad
        self._inst = inst

        flags = 0
        for t in terms:
            flags |= {"pgrad": native.TERM_PGRAD, "avisc": native.TERM_AVISC,
                      "xsph": native.TERM_XSPH}[t]
        rec = native.BatchRecipe()
        rec.dim = self.dim
        rec.subdiv = per_inst[0]
        rec.margin = float(margin)
        rec.scheme = {"euler": 0, "rk2": 1}[integrator]
        rec.list_cap = int(list_cap)
        rec.radius_scale = radius_scale
        rec.dt = self.dt
        rec.density = native.DensityParams(dim=self.dim, tait=1, co=co, ro=ro, gamma=gamma)
        rec.term = native.SourceTerm(src=0, flags=flags, alpha=alpha, beta=beta, eta=0.0,
                                     eps=eps, delp=1.0)
        g = gravity or (0.0, 0.0, 0.0)
        rec.rates = native.RatesParams(dim=self.dim, add_velocity=1 if step_positions else 0,
                                       gx=g[0], gy=g[1], gz=g[2],
                                       add_gravity=1 if gravity else 0)
        self.recipe = rec
        L = native.lib()
        h = ctypes.c_void_p()
        native.check(L.sph_batch_create(ctypes.byref(h)), "sph_batch_create")
        self._b = h
        torch.cuda.synchronize()
        native.check(L.sph_batch_setup(h, ctypes.byref(view), inst, ninst, ctypes.byref(rec)),
                     "sph_batch_setup")
        self.steps = 0

    @classmethod
    def from_solvers(cls, solvers, dt, **kw):
        """Batch already configured single-array solvers (``(solver,
        particles)`` pairs) that share one recipe: SPHRho + Tait, then
        integrating PGrad / AV / XSPH / gravity / position stepping."""
        first = solvers[0][0].integrator
        stages = [type(st).__name__ for st in first.stages]
        if stages != ["DensityStage", "RatesStage"] or first.stages[0].tait is None:
            raise NotImplementedError("batches need the recipe SPHRho+Tait, then rate terms")
        dens, rates = first.stages
        t = dens.tait.funcs[0]
        terms = sorted(rates.terms[0]["kinds"]) if rates.terms else []
        p0 = rates.terms[0] if rates.terms else {}
        integ = {"EulerIntegrator": "euler", "RK2Integrator": "rk2"}[type(first).__name__]
        instances = []
        for solver, particles in solvers:
            st = solver.integrator.stages
            if [type(x).__name__ for x in st] != stages:
                raise ValueError("every solver of a batch must have the same recipe")
            pa = particles.arrays[0]
            instances.append({k: pa.get(k) for k in PROPS if pa.has_array(k)})
        return cls(instances, dim=dens.calc.kernel.dim, dt=dt, co=t.co, ro=t.ro, gamma=t.gamma,
                   terms=terms, alpha=p0.get("alpha", 0.0), beta=p0.get("beta", 0.0),
                   eps=p0.get("eps", 0.5), gravity=rates.gravity,
                   step_positions=rates.add_velocity, integrator=integ, **kw)

    def step(self, nsteps=1, check=True):
        """Advance every instance by ``nsteps`` steps; check the error word."""
        L = native.lib()
        torch.cuda.current_stream().synchronize()
        native.check(L.sph_batch_step(self._b, int(nsteps), 1 if self.use_graph else 0),
                     "sph_batch_step")
        self.steps += nsteps
        if check:
            self.check()

    def stats(self):
        """Regions re-derived so far, cells of the current grids, steps
        completed, groups of equal subdivision."""
        out = (ctypes.c_int64 * 4)()
        native.check(native.lib().sph_batch_stats(self._b, out), "sph_batch_stats")
        return {"regrids": out[0], "cells": out[1], "steps": out[2], "groups": out[3]}

    def stream(self):
        """The batch's CUDA stream as a torch stream (for events)."""
        h = ctypes.c_void_p()
        native.check(native.lib().sph_batch_stream(self._b, ctypes.byref(h)), "batch stream")
        return torch.cuda.ExternalStream(h.value)

    def pair_counts(self):
        """Neighbour pairs (incl. self) per instance in the last evaluation."""
        out = (ctypes.c_uint64 * self.ninstances)()
        native.check(native.lib().sph_batch_pair_counts(self._b, out), "pair counts")
        return np.array(out[:], dtype=np.int64)

    def sync(self):
        native.check(native.lib().sph_batch_sync(self._b), "sph_batch_sync")

    def check(self):
        w = ctypes.c_uint32()
        native.check(native.lib().sph_batch_error_word(self._b, ctypes.byref(w)), "error word")
        if w.value & native.SPH_EFLAG_JUMP:
            raise RuntimeError("Particle moved by more than one cell width")
        if w.value & native.SPH_EFLAG_BOX:
            raise RuntimeError("a particle left its instance's grid region (margin 0)")

    def set(self, **props):
        """Overwrite whole concatenated properties (all instances, in
        instance order) from host or device tensors / arrays.  Waits for the
        batch's own stream first (a step may still be using the arrays);
        copies from page-locked host memory run asynchronously, all of them
        before one synchronisation."""
        self.sync()
        for name, val in props.items():
            if name not in self.arrays:
                raise ValueError("unknown batch property %r" % name)
            t = torch.as_tensor(val)
            if t.numel() != self.n:
                raise ValueError("property %r needs %d values" % (name, self.n))
            self.arrays[name].copy_(t.reshape(-1), non_blocking=True)
        torch.cuda.current_stream().synchronize()

    # -- staged host transfers (see pysph_gb300.base.transfer) -----------------
    def _torch_stream(self):
        s = getattr(self, "_tstream", None)
        if s is None:
            s = self._tstream = self.stream()
        return s

    def upload(self, **props):
        """Start copying whole concatenated properties from host memory
        (page-locked for an asynchronous copy) on a copy stream; returns at
        once.  Page-locked sources must stay unchanged until ``set_staged``."""
        for name in props:
            if name not in self.arrays:
                raise ValueError("unknown batch property %r" % name)
        up = transfer.upload_tensors(self.arrays, props, self.n)
        up.pa = self
        return up

    def set_staged(self, up):
        """``set`` with the values of an earlier ``upload``: the batch's
        stream waits for its copies and takes them over on the device (no
        host synchronisation)."""
        if not isinstance(up, transfer.StagedUpload) or up.pa is not self:
            raise ValueError("set_staged takes an upload of this batch")
        transfer.apply_staged(self.arrays, up, self._torch_stream())

    def download(self, *props):
        """Start reading whole concatenated properties back: a device
        snapshot on the batch's stream, copied to page-locked host memory on
        a copy stream.  ``result()`` of the returned object waits for those
        copies only."""
        for name in props:
            if name not in self.arrays:
                raise ValueError("unknown batch property %r" % name)
        return transfer.download_tensors({p: self.arrays[p] for p in props}, props,
                                         self._torch_stream())

    def _host(self, tensors):
        """Host copies through page-locked buffers, one synchronisation."""
        out = []
        for t in tensors:
            h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
            h.copy_(t, non_blocking=True)
            out.append(h)
        torch.cuda.current_stream().synchronize()
        return [h.numpy() for h in out]

    def get_all(self, *props):
        """Whole concatenated properties as NumPy arrays (synchronises)."""
        self.sync()
        out = self._host([self.arrays[p] for p in props])
        return out[0] if len(out) == 1 else tuple(out)

    def get(self, k, *props):
        """Properties of instance ``k`` as NumPy arrays (synchronises)."""
        self.sync()
        a, b = int(self.offsets[k]), int(self.offsets[k + 1])
        out = self._host([self.arrays[p][a:b] for p in props])
        return out[0] if len(out) == 1 else tuple(out)

    @property
    def ninstances(self):
        return len(self.offsets) - 1

    def __del__(self):
        b = getattr(self, "_b", None)
        if b is not None:
            try:
                native.load_library(False).sph_batch_destroy(b)
            except Exception:
                pass
