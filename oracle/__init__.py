"""CPU oracle for the SPH particle-step hot path -- TEST INFRASTRUCTURE.

The oracle is the checker the GPU path is compared with.  It restates the
reference PySPH algorithm in FP64 (``oracle/sph_oracle.c`` for the
neighbour search and pair sums; the integrator bookkeeping below) and is
pinned against the golden fixtures that the reference itself produced
(``tests/golden``).  Only tests, ``__graft_entry__.smoke()`` and the CPU
baseline of ``bench.py`` may import it; the product never does.

Reference routines restated here (paths relative to ``source/pysph``):

* ``solver/integrator.py:229-912`` -- calc bookkeeping, Euler, RK2, RK4,
  predictor-corrector and leap-frog steps (``Problem.integrate_*``);
* ``sph/sph_calc.pyx:223-276`` -- zero the outputs, then sum over sources
  (``Problem._run_op``);
* the per-function pair sums and the neighbour search -- see the C file.
"""
import ctypes
import math
import os
import platform
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(HERE, "sph_oracle.c")
_BUILD = os.path.join(HERE, "_build")
_LIB = os.path.join(_BUILD, "libsph_oracle_%s.so" % platform.machine())
_lock = threading.Lock()
_lib = None


def build(force=False):
    """Compile the C restatement (gcc, OpenMP, no FMA contraction)."""
    os.makedirs(_BUILD, exist_ok=True)
    if (not force and os.path.exists(_LIB)
            and os.path.getmtime(_LIB) >= os.path.getmtime(_SRC)):
        return _LIB
    tmp = _LIB + ".%d.tmp" % os.getpid()
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", _SRC, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB)
    return _LIB


class OrcArray(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64)] + [
        (name, ctypes.c_void_p) for name in
        ("x", "y", "z", "u", "v", "w", "m", "h", "rho", "p", "cs",
         "nx", "ny", "nz", "tx", "ty", "tz", "tag")]


def lib():
    global _lib
    with _lock:
        if _lib is None:
            L = ctypes.CDLL(build())
            P = ctypes.POINTER(OrcArray)
            d = ctypes.c_double
            vp = ctypes.c_void_p
            i = ctypes.c_int
            L.orc_neighbors.restype = ctypes.c_int64
            L.orc_neighbors.argtypes = [P, P, d, d, i, vp, vp]
            L.orc_neighbor_digest.restype = ctypes.c_int64
            L.orc_neighbor_digest.argtypes = [P, P, d, d, vp, vp]
            L.orc_neighbors_varh.restype = ctypes.c_int64
            L.orc_neighbors_varh.argtypes = [P, P, d, d, i, vp, vp]
            L.orc_sph_rho.argtypes = [P, P, vp, vp, i, vp]
            L.orc_tait.argtypes = [P, d, d, d, vp, vp]
            L.orc_pgrad.argtypes = [P, P, vp, vp, i, i, vp, vp, vp]
            L.orc_avisc.argtypes = [P, P, vp, vp, i, d, d, d, vp, vp, vp]
            L.orc_xsph.argtypes = [P, P, vp, vp, i, d, i, vp, vp, vp]
            L.orc_momentum.argtypes = [P, P, vp, vp, i, d, d, d, i, vp, vp, vp]
            L.orc_drho.argtypes = [P, P, vp, vp, i, vp]
            L.orc_pilot_rho.argtypes = [P, P, vp, vp, i, d, vp]
            L.orc_vdiv.argtypes = [P, P, vp, vp, i, vp]
            L.orc_bforce.argtypes = [P, P, vp, vp, d, vp, vp, vp]
            L.orc_const3.argtypes = [P, d, d, d, i, vp, vp, vp]
            L.orc_position_stepping.argtypes = [P, i, vp, vp, vp]
            L.orc_cubic_w.restype = d
            L.orc_cubic_w.argtypes = [i] + [d] * 7
            L.orc_cubic_grad.argtypes = [i] + [d] * 7 + [vp]
            L.orc_num_threads.restype = i
            _lib = L
    return _lib


def num_threads():
    return lib().orc_num_threads()


def _ptr(a):
    return None if a is None else a.ctypes.data


class _Arr:
    """Keeps the numpy buffers alive while an OrcArray points at them."""

    def __init__(self, props):
        n = len(props["x"])
        self.keep = {}
        st = OrcArray()
        st.n = n
        for name, _ in OrcArray._fields_[1:]:
            a = props.get(name)
            if a is not None:
                a = np.ascontiguousarray(a, dtype=np.int64 if name == "tag" else np.float64)
                self.keep[name] = a
            setattr(st, name, _ptr(a))
        self.st = st
        self.ref = ctypes.byref(st)


def cubic_w(dim, a, b, h):
    return lib().orc_cubic_w(dim, *a, *b, h)


def cubic_grad(dim, a, b, h):
    g = np.zeros(3)
    lib().orc_cubic_grad(dim, *a, *b, h, g.ctypes.data)
    return g


def neighbors(dst, src, cell_size, radius_scale=2.0, same=False, variable_h=False):
    """CSR neighbour lists (ascending source index, then with ``same`` the
    destination swapped with the last entry, nnps.pyx:609-616);
    ``variable_h`` gives the symmetric relation of VarHNbrParticleLocator."""
    D, S = _Arr(dst), _Arr(src)
    n = D.st.n
    fn = lib().orc_neighbors_varh if variable_h else lib().orc_neighbors
    offsets = np.zeros(n + 1, np.int64)
    fn(D.ref, S.ref, cell_size, radius_scale, int(same), offsets.ctypes.data, None)
    np.cumsum(offsets, out=offsets)
    index = np.zeros(max(int(offsets[-1]), 1), np.int64)
    fn(D.ref, S.ref, cell_size, radius_scale, int(same), offsets.ctypes.data, index.ctypes.data)
    return offsets, index[: offsets[-1]]


def mix64(j):
    """The splitmix64 finaliser of sph_oracle.c, elementwise over uint64."""
    z = np.asarray(j).astype(np.uint64) + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def neighbor_digest(dst, src, cell_size, radius_scale=2.0):
    """Per destination: neighbour count and the wrap-around sum of mix64 over
    its source indices (an order-independent digest of the set), without
    storing the lists."""
    D, S = _Arr(dst), _Arr(src)
    n = D.st.n
    counts = np.zeros(n + 1, np.int64)
    digest = np.zeros(max(n, 1), np.uint64)
    lib().orc_neighbor_digest(D.ref, S.ref, cell_size, radius_scale, counts.ctypes.data,
                              digest.ctypes.data)
    return counts[1:], digest[:n]


def pair_sum(kind, dst, src, offsets, index, dim, params=None, nout=3):
    """Evaluate one SPH function from explicit neighbour lists.

    Returns a list of ``nout`` FP64 arrays (zero-initialised, then summed,
    like ``SPHCalc.sph``)."""
    params = params or {}
    D, S = _Arr(dst), _Arr(src)
    n = D.st.n
    outs = [np.zeros(n) for _ in range(3)]
    o = [x.ctypes.data for x in outs]
    off = np.ascontiguousarray(offsets, np.int64)
    idx = np.ascontiguousarray(index, np.int64)
    L = lib()
    if kind == "rho":
        L.orc_sph_rho(D.ref, S.ref, off.ctypes.data, idx.ctypes.data, dim, o[0])
        return outs[:1]
    if kind == "drho":
        L.orc_drho(D.ref, S.ref, off.ctypes.data, idx.ctypes.data, dim, o[0])
        return outs[:1]
    if kind == "pilotrho":
        L.orc_pilot_rho(D.ref, S.ref, off.ctypes.data, idx.ctypes.data, dim,
                        ctypes.c_double(params["h0"]), o[0])
        return outs[:1]
    if kind == "vdiv":
        L.orc_vdiv(D.ref, S.ref, off.ctypes.data, idx.ctypes.data, dim, o[0])
        return outs[:1]
    if kind == "pgrad":
        L.orc_pgrad(D.ref, S.ref, off.ctypes.data, idx.ctypes.data, dim, nout, *o)
    elif kind == "avisc":
        L.orc_avisc(D.ref, S.ref, off.ctypes.data, idx.ctypes.data, dim,
                    params.get("alpha", 1.0), params.get("beta", 1.0), 0.0, *o)
    elif kind == "momentum":
        L.orc_momentum(D.ref, S.ref, off.ctypes.data, idx.ctypes.data, dim,
                       params.get("alpha", 1.0), params.get("beta", 1.0),
                       params.get("eta", 0.1), nout, *o)
    elif kind == "xsph":
        L.orc_xsph(D.ref, S.ref, off.ctypes.data, idx.ctypes.data, dim,
                   params.get("eps", 0.5), nout, *o)
    elif kind == "bforce":
        L.orc_bforce(D.ref, S.ref, off.ctypes.data, idx.ctypes.data,
                     params.get("delp", 1.0), *o)
    else:
        raise ValueError(kind)
    return outs[:nout]


def adke_smoothing(dst, h0, k=1.0, eps=0.0, nreal=None):
    """ADKESmoothingUpdate.eval (sph/funcs/adke_funcs.pyx:118-147): new h of
    the LocalReal particles (0 for the others, which SPHCalc.sph zeroes);
    the logarithms are summed in index order as the reference's loop does."""
    rhop = np.asarray(dst["rhop"], np.float64)
    n = rhop.size
    tag = np.asarray(dst.get("tag", np.zeros(n, np.int64)))
    nreal = n if nreal is None else nreal
    log_g = 0.0
    for i in range(n):
        if tag[i] == 0:
            log_g += math.log(rhop[i])
    log_g /= nreal
    g = math.exp(log_g)
    out = np.zeros(n)
    for i in range(n):
        if tag[i] == 0:
            out[i] = h0 * k * (g / rhop[i]) ** eps
    return out


def adke_conduction(dst, g1, g2, nreal=None):
    """ADKEConductionCoeffUpdate.eval (adke_funcs.pyx:256-291):
    q = (g1 cs + g2 h (|div| - div)) h over the LocalReal particles among the
    first nreal (0 for the others)."""
    h = np.asarray(dst["h"], np.float64)
    n = h.size
    tag = np.asarray(dst.get("tag", np.zeros(n, np.int64)))
    cs = np.asarray(dst["cs"], np.float64)
    div = np.asarray(dst["div"], np.float64)
    nreal = n if nreal is None else nreal
    out = np.zeros(n)
    for i in range(nreal):
        if tag[i] == 0:
            o = g1 * cs[i] + (g2 * h[i] * (abs(div[i]) - div[i]))
            out[i] = o * h[i]
    return out


def tait(dst, co, ro, gamma=7.0):
    D = _Arr(dst)
    p = np.zeros(D.st.n)
    cs = np.zeros(D.st.n)
    lib().orc_tait(D.ref, co, ro, gamma, p.ctypes.data, cs.ctypes.data)
    return p, cs


def periodic_images(src, xmin, xmax, reach):
    """Ghost copies for a domain periodic in x (base/cell.pyx:1277-1376): the
    particles within ``reach`` of either end, copied with x shifted by
    +-(xmax - xmin) (FP64 adds, as the reference shifts its ghosts) and the
    rest of their state unchanged.  Returns (extended property dict, origin
    index of every ghost).  The reference copies whole cells of size 2 max h
    whose faces lie within reach; the extra copies lie beyond every search
    radius, so the neighbour sets are the same.  Particles that have left
    the period (x is never wrapped) widen the reach by their overshoot, so
    every particle sees the nearest image of every other (the reference's
    binning wraps such particles once and misses images beyond its cells)."""
    L = xmax - xmin
    x = np.asarray(src["x"], np.float64)
    if x.size:
        reach = reach + max(0.0, float(x.max()) - xmax, xmin - float(x.min()))
    lo = np.nonzero(x - xmin < reach)[0]
    hi = np.nonzero(xmax - x < reach)[0]
    origin = np.concatenate([lo, hi]).astype(np.int64)
    shift = np.concatenate([np.full(lo.size, L), np.full(hi.size, -L)])
    ext = {}
    for k, v in src.items():
        v = np.asarray(v)
        ext[k] = np.concatenate([v, v[origin]])
    ext["x"] = np.concatenate([x, x[origin] + shift])
    if "tag" in ext:
        ext["tag"][len(x):] = 0
    return ext, origin


# ---------------------------------------------------------------------------
# Problem: a set of particle arrays plus an ordered list of operations,
# stepped exactly like solver/integrator.py steps its calcs.
# ---------------------------------------------------------------------------

class Op:
    """One calc: ``kind`` in rho | tait | pgrad | avisc | momentum | drho |
    xsph | bforce | gravity | step, on destination ``dest`` from
    ``sources``."""

    # the function tags of the reference (sph/funcs/*.pyx ``self.tag``)
    TAGS = {"rho": "density", "drho": "density", "tait": "state", "pgrad": "velocity",
            "avisc": "velocity", "momentum": "velocity", "bforce": "velocity",
            "gravity": "velocity", "step": "position", "xsph": "position",
            "pilotrho": "pilotrho", "adke_h": "h", "vdiv": "vdivergence", "adke_q": "q"}

    def __init__(self, kind, dest, updates, sources=(), integrates=False, **params):
        self.kind = kind
        self.dest = dest
        self.sources = list(sources)
        self.updates = list(updates)
        self.integrates = integrates
        self.params = params
        self.tag = self.TAGS[kind]


class Problem:
    def __init__(self, arrays, ops, dim, radius_scale=2.0, variable_h=False, periodic=None):
        # arrays: dict name -> dict of float64 property arrays (copied)
        self.arrays = {}
        for name, props in arrays.items():
            n = len(props["x"])
            a = {k: np.array(v, dtype=np.int64 if k == "tag" else np.float64)
                 for k, v in props.items()}
            for k, default in (("y", 0.0), ("z", 0.0), ("u", 0.0), ("v", 0.0),
                               ("w", 0.0), ("m", 1.0), ("h", 1.0), ("p", 0.0),
                               ("rho", 1.0), ("cs", 0.0), ("e", 0.0)):
                if k not in a:
                    a[k] = np.full(n, default)
            self.arrays[name] = a
        self.ops = ops
        self.dim = dim
        self.radius_scale = radius_scale
        self.variable_h = variable_h
        # (xmin, xmax) of a domain periodic in x, or None
        self.periodic = periodic
        max_h = max(float(a["h"].max()) for a in self.arrays.values() if a["h"].size)
        # CellManager.compute_cell_size: base/cell.pyx:893-925
        self.cell_size = radius_scale * max_h
        self.k = {}
        self.nbr_cache = {}

    def _source(self, src):
        """The source arrays a pair pass sees: with a periodic domain, the
        particles plus their ghost images (state as it is now)."""
        a = self.arrays[src]
        if self.periodic is None:
            return a, None
        reach = self.radius_scale * max(float(b["h"].max()) for b in self.arrays.values())
        return periodic_images(a, self.periodic[0], self.periodic[1], reach * (1 + 1e-12))

    def neighbours(self, dest, src):
        key = (dest, src)
        if key not in self.nbr_cache:
            ext, _ = self._source(src)
            self.nbr_cache[key] = neighbors(self.arrays[dest], ext, self.cell_size,
                                            self.radius_scale, same=(dest == src),
                                            variable_h=self.variable_h)
        return self.nbr_cache[key]

    def _moved(self):
        self.nbr_cache = {}

    def _run_op(self, op):
        """Evaluate one calc; returns its outputs (list, one per update)."""
        d = self.arrays[op.dest]
        nout = len(op.updates)
        n = len(d["x"])
        outs = [np.zeros(n) for _ in range(nout)]
        if op.kind == "tait":
            p, cs = tait(d, op.params["co"], op.params["ro"], op.params.get("gamma", 7.0))
            return [p, cs]
        if op.kind == "adke_h":
            return [adke_smoothing(d, op.params["h0"], op.params.get("k", 1.0),
                                   op.params.get("eps", 0.0))]
        if op.kind == "adke_q":
            return [adke_conduction(d, op.params.get("g1", 0.0), op.params.get("g2", 0.0))]
        if op.kind == "gravity":
            D = _Arr(d)
            tmp = [np.zeros(n) for _ in range(3)]
            lib().orc_const3(D.ref, op.params.get("gx", 0.0), op.params.get("gy", 0.0),
                             op.params.get("gz", 0.0), nout, *[t.ctypes.data for t in tmp])
            return tmp[:nout]
        if op.kind == "step":
            D = _Arr(d)
            tmp = [np.zeros(n) for _ in range(3)]
            lib().orc_position_stepping(D.ref, nout, *[t.ctypes.data for t in tmp])
            return tmp[:nout]
        for s in op.sources:
            off, idx = self.neighbours(op.dest, s)
            res = pair_sum(op.kind, d, self._source(s)[0], off, idx, self.dim, op.params, nout)
            for o, r in zip(outs, res):
                o += r
        return outs

    # integrator.py:432-470
    def eval(self, kname, only=None):
        for ci, op in enumerate(self.ops):
            if only is not None and ci not in only:
                continue
            res = self._run_op(op)
            if op.integrates:
                self.k[(kname, ci)] = res
            else:
                for upd, r in zip(op.updates, res):
                    self.arrays[op.dest][upd] = r
                if "h" in op.updates:
                    # new smoothing lengths: the calc re-bins (sph_calc.pyx:
                    # 262-263 after adke_funcs.pyx:145-147)
                    self._moved()

    def _integrating(self):
        return [(ci, op) for ci, op in enumerate(self.ops) if op.integrates]

    # integrator.py:339-367
    def _set_initial(self):
        init = {}
        for ci, op in self._integrating():
            for upd in op.updates:
                init[(op.dest, upd)] = self.arrays[op.dest][upd].copy()
        return init

    # integrator.py:525-573
    def integrate_euler(self, dt):
        init = self._set_initial()
        self.eval("k1")
        for ci, op in self._integrating():
            for j, upd in enumerate(op.updates):
                updated = init[(op.dest, upd)] + self.k[("k1", ci)][j] * dt
                self.arrays[op.dest][upd] = updated
                init[(op.dest, upd)] = updated
        self._moved()

    # integrator.py:581-645
    def integrate_rk2(self, dt):
        init = self._set_initial()
        self.eval("k1")
        for (dest, upd), a in init.items():
            self.arrays[dest][upd] = a.copy()
        for ci, op in self._integrating():
            for j, upd in enumerate(op.updates):
                cur = self.arrays[op.dest][upd]
                self.arrays[op.dest][upd] = cur + self.k[("k1", ci)][j] * dt
        self._moved()
        self.eval("k2")
        for ci, op in self._integrating():
            for j, upd in enumerate(op.updates):
                updated = init[(op.dest, upd)] + 0.5 * dt * (
                    self.k[("k1", ci)][j] + self.k[("k2", ci)][j])
                self.arrays[op.dest][upd] = updated
                init[(op.dest, upd)] = updated
        self._moved()


    # integrator.py:369-430 reset_current_arrays + step, for the ops in ``only``
    def _reset_and_step(self, init, kname, dt, only=None):
        sel = [(ci, op) for ci, op in self._integrating() if only is None or ci in only]
        for ci, op in sel:
            for upd in op.updates:
                self.arrays[op.dest][upd] = init[(op.dest, upd)].copy()
        for ci, op in sel:
            for j, upd in enumerate(op.updates):
                cur = self.arrays[op.dest][upd]
                self.arrays[op.dest][upd] = cur + self.k[(kname, ci)][j] * dt

    # integrator.py:650-730
    def integrate_rk4(self, dt):
        init = self._set_initial()
        for kname, h in (("k1", 0.5 * dt), ("k2", 0.5 * dt), ("k3", dt)):
            self.eval(kname)
            self._reset_and_step(init, kname, h)
            self._moved()
        self.eval("k4")
        for ci, op in self._integrating():
            for j, upd in enumerate(op.updates):
                k1, k2, k3, k4 = (self.k[(kn, ci)][j] for kn in ("k1", "k2", "k3", "k4"))
                updated = init[(op.dest, upd)] + (dt / 6.0) * (k1 + 2 * k2 + 2 * k3 + k4)
                self.arrays[op.dest][upd] = updated
                init[(op.dest, upd)] = updated
        self._moved()

    # integrator.py:734-796
    def integrate_pc(self, dt):
        init = self._set_initial()
        for kname in ("k1", "k2"):
            self.eval(kname)
            self._reset_and_step(init, kname, 0.5 * dt)
            self._moved()
        for ci, op in self._integrating():
            for upd in op.updates:
                updated = 2 * self.arrays[op.dest][upd] - init[(op.dest, upd)]
                self.arrays[op.dest][upd] = updated
                init[(op.dest, upd)] = updated
        self._moved()

    # integrator.py:802-912
    def integrate_leapfrog(self, dt):
        init = self._set_initial()
        ncalcs = {ci for ci, op in enumerate(self.ops) if op.tag != "position"}
        pcalcs = [ci for ci, op in enumerate(self.ops) if op.tag == "position"]
        icalcs = [ci for ci, op in self._integrating() if op.tag != "position"]
        self.eval("k1", ncalcs)
        self._reset_and_step(init, "k1", dt, ncalcs)
        self.eval("k1", set(pcalcs))
        self._reset_and_step(init, "k1", dt, set(pcalcs))
        # add_correction_for_position (:841-872)
        pos = self.ops[pcalcs[0]]
        for ci in icalcs:
            op = self.ops[ci]
            if op.tag != "velocity":
                continue
            for j in range(len(op.updates)):
                upd = pos.updates[j]
                cur = self.arrays[pos.dest][upd]
                self.arrays[pos.dest][upd] = cur + 0.5 * dt * dt * self.k[("k1", ci)][j]
        self._moved()
        self.eval("k2", ncalcs)
        for ci in icalcs:
            op = self.ops[ci]
            for j, upd in enumerate(op.updates):
                cur = self.arrays[op.dest][upd]
                self.arrays[op.dest][upd] = cur + 0.5 * dt * (
                    self.k[("k2", ci)][j] - self.k[("k1", ci)][j])


# ---------------------------------------------------------------------------
# operation lists matching pysph_gb300.workloads.setup_* (same order, same
# parameters), expressed independently of the product's solver classes.
# ---------------------------------------------------------------------------

def drop_ops(c0=1400.0, rho0=1.0, alpha=0.01, beta=0.0, eps=0.5):
    return [
        Op("rho", "fluid", ["rho"], ["fluid"]),
        Op("tait", "fluid", ["p", "cs"], co=c0, ro=rho0),
        Op("pgrad", "fluid", ["u", "v"], ["fluid"], integrates=True),
        Op("avisc", "fluid", ["u", "v", "w"], ["fluid"], integrates=True, alpha=alpha, beta=beta),
        Op("step", "fluid", ["x", "y"], integrates=True),
        Op("xsph", "fluid", ["x", "y"], ["fluid"], integrates=True, eps=eps),
    ]


def dam_ops(dx, c0, rho0=1000.0, alpha=0.1, beta=0.0, g=-9.81):
    return [
        Op("tait", "fluid", ["p", "cs"], co=c0, ro=rho0),
        Op("rho", "fluid", ["rho"], ["fluid"]),
        Op("pgrad", "fluid", ["u", "v"], ["fluid"], integrates=True),
        Op("avisc", "fluid", ["u", "v", "w"], ["fluid"], integrates=True, alpha=alpha, beta=beta),
        Op("bforce", "fluid", ["u", "v", "w"], ["boundary"], integrates=True, delp=dx),
        Op("gravity", "fluid", ["u", "v", "w"], integrates=True, gy=g),
        Op("step", "fluid", ["x", "y"], integrates=True),
    ]


def cube_ops(c0=1.0, rho0=1.0, alpha=0.1, beta=0.0):
    return [
        Op("rho", "fluid", ["rho"], ["fluid"]),
        Op("tait", "fluid", ["p", "cs"], co=c0, ro=rho0),
        Op("pgrad", "fluid", ["u", "v", "w"], ["fluid"], integrates=True),
        Op("avisc", "fluid", ["u", "v", "w"], ["fluid"], integrates=True, alpha=alpha, beta=beta),
        Op("step", "fluid", ["x", "y", "z"], integrates=True),
    ]


def fluid_ops(c0=100.0, ro=1.0, alpha=0.01, beta=0.0, eta=0.1, eps=0.1):
    """solver/fluid_solver.py:51-83 (FluidSolver): Tait, continuity density
    rate, MomentumEquation, position stepping, XSPH."""
    return [
        Op("tait", "fluid", ["p", "cs"], co=c0, ro=ro),
        Op("drho", "fluid", ["rho"], ["fluid"], integrates=True),
        Op("momentum", "fluid", ["u", "v", "w"], ["fluid"], integrates=True, alpha=alpha,
           beta=beta, eta=eta),
        Op("step", "fluid", ["x", "y"], integrates=True),
        Op("xsph", "fluid", ["x", "y"], ["fluid"], integrates=True, eps=eps),
    ]
