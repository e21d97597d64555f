"""Launch helpers shared by ``SPHCalc`` and the integrators.

Each helper validates its arguments, makes the cell manager's snapshots
current and calls one entry point of the C ABI (``include/pysph_gb300.h``)
on the current torch stream.  Outputs are FP64 device tensors of the
destination array.
"""
import ctypes

import torch

from .. import native
from ..base.cell import SNAPSHOT_PROPS, array_view

RATE_TERM = {"pgrad": native.TERM_PGRAD, "avisc": native.TERM_AVISC,
             "xsph": native.TERM_XSPH, "bforce": native.TERM_BFORCE,
             "momentum": native.TERM_PGRAD | native.TERM_AVISC, "drho": native.TERM_DRHO,
             "vdiv": native.TERM_VDIV}


def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _vp_array(ts):
    arr = (ctypes.c_void_p * 3)()
    for i in range(3):
        t = ts[i] if i < len(ts) else None
        arr[i] = None if t is None else t.data_ptr()
    return arr


def note_written(cm, pa, names, consistent=False):
    """Record that ``names`` of ``pa`` were written on the device."""
    if any(n in SNAPSHOT_PROPS for n in names if n):
        pa.touch()
        if consistent:
            cm.mark_fresh(pa)


def nbr_lists(cm, dest, sources):
    """Build the neighbour lists of ``dest`` among ``sources`` (if stale)."""
    cm.ensure_current()
    L = native.lib()
    srcs = (ctypes.c_int * max(1, len(sources)))(*[cm.slot(s) for s in sources])
    native.check(L.sph_nbr_lists(cm.context(), cm.slot(dest), srcs, len(sources)), "lists")


def density(cm, dest, sources, dim, rho_out, tait=None, p_out=None, cs_out=None, h0=0.0):
    """Summation density of ``dest`` from ``sources`` into ``rho_out``;
    with ``tait=(co, ro, gamma)`` also p and cs; with ``h0 > 0`` the kernel
    at that fixed h (the ADKE pilot density)."""
    cm.ensure_current()
    L = native.lib()
    ctx = cm.context()
    srcs = (ctypes.c_int * max(1, len(sources)))(*[cm.slot(s) for s in sources])
    prm = native.DensityParams(dim=int(dim), tait=1 if tait else 0,
                               co=tait[0] if tait else 0.0, ro=tait[1] if tait else 1.0,
                               gamma=tait[2] if tait else 7.0, h0=float(h0))
    native.check(L.sph_density(ctx, cm.slot(dest), srcs, len(sources), ctypes.byref(prm),
                               _p(rho_out), _p(p_out), _p(cs_out)), "SPHRho")


def rates(cm, dest, terms, dim, acc=(), pos=(), accumulate=False, gravity=None,
          add_velocity=False, drho=None):
    """One launch of the rates kernel.  ``terms``: list of dicts with keys
    src (ParticleArray), kinds (set of pgrad/avisc/xsph/bforce) and the
    function parameters."""
    cm.ensure_current()
    L = native.lib()
    ctx = cm.context()
    n = len(terms)
    if n > native.MAX_SOURCES:
        raise NotImplementedError("more than %d source terms in one rates launch" % native.MAX_SOURCES)
    arr = (native.SourceTerm * max(1, n))()
    for i, t in enumerate(terms):
        flags = 0
        for k in t["kinds"]:
            flags |= RATE_TERM[k]
        arr[i] = native.SourceTerm(src=cm.slot(t["src"]), flags=flags,
                                   alpha=t.get("alpha", 0.0), beta=t.get("beta", 0.0),
                                   eta=t.get("eta", 0.0), eps=t.get("eps", 0.0),
                                   delp=t.get("delp", 1.0))
    g = gravity or (0.0, 0.0, 0.0)
    prm = native.RatesParams(dim=int(dim), add_velocity=1 if add_velocity else 0,
                             gx=g[0], gy=g[1], gz=g[2], add_gravity=1 if gravity else 0,
                             drho_out=None if drho is None else drho.data_ptr())
    native.check(L.sph_rates(ctx, cm.slot(dest), arr, n, ctypes.byref(prm), _vp_array(acc),
                             _vp_array(pos), 1 if accumulate else 0), "rates")


def tait(cm, dest, co, ro, gamma, p_out, cs_out):
    L = native.lib()
    ctx = cm.context()
    native.check(L.sph_tait(ctx, dest.get_number_of_particles(), _p(dest.get_device("rho")),
                            _p(dest.get_device("tag")), co, ro, gamma, _p(p_out), _p(cs_out)),
                 "TaitEquation")


def _prop(pa, name, why):
    if not pa.has_array(name):
        raise AttributeError("%s needs property %s of %s" % (why, name, pa.name))
    return pa.get_device(name)


def adke_smoothing(cm, dest, h0, k, eps, h_out):
    """ADKESmoothingUpdate: h_out of the LocalReal particles from ``rhop``."""
    ctx = cm.context()
    rhop = _prop(dest, "rhop", "ADKESmoothingUpdate")
    native.check(native.lib().sph_adke_smoothing(
        ctx, dest.get_number_of_particles(), dest.num_real_particles,
        _p(dest.get_device("tag")), _p(rhop), h0, k, eps, _p(h_out)), "ADKESmoothingUpdate")


def adke_conduction(cm, dest, g1, g2, q_out):
    """ADKEConductionCoeffUpdate: q_out of the LocalReal particles."""
    ctx = cm.context()
    args = [_prop(dest, p, "ADKEConductionCoeffUpdate") for p in ("cs", "h", "div")]
    native.check(native.lib().sph_adke_conduction(
        ctx, dest.num_real_particles, _p(dest.get_device("tag")), *[_p(a) for a in args],
        g1, g2, _p(q_out)), "ADKEConductionCoeffUpdate")


def const_rates(cm, dest, kind, outs, g=None):
    """kind 0: outs = g (gravity); kind 1: outs = (u, v, w) (position stepping)."""
    L = native.lib()
    ctx = cm.context()
    g3 = (ctypes.c_double * 3)(*(g or (0.0, 0.0, 0.0)))
    u, v, w = (dest.get_device(c) if dest.has_array(c) else None for c in ("u", "v", "w"))
    native.check(L.sph_const_rates(ctx, kind, dest.get_number_of_particles(),
                                   _p(dest.get_device("tag")), g3, _p(u), _p(v), _p(w),
                                   len(outs), _vp_array(outs)), "const rates")


def axpy(cm, n, lines):
    """``lines``: list of (out, save, base, k1, k2, c1, mode[, k3, k4]) device
    tensors (modes as ``sph_axpy_line`` in the C header)."""
    if not lines:
        return
    L = native.lib()
    ctx = cm.context()

    def ptr(t):
        return None if t is None else t.data_ptr()

    for start in range(0, len(lines), native.MAX_AXPY_LINES):
        chunk = lines[start:start + native.MAX_AXPY_LINES]
        arr = (native.AxpyLine * len(chunk))()
        for i, line in enumerate(chunk):
            out, save, base, k1, k2, c1, mode = line[:7]
            k3, k4 = (line[7], line[8]) if len(line) > 7 else (None, None)
            arr[i] = native.AxpyLine(out=out.data_ptr(), save=ptr(save), base=base.data_ptr(),
                                     k1=ptr(k1), k2=ptr(k2), c1=float(c1), mode=int(mode),
                                     k3=ptr(k3), k4=ptr(k4))
        native.check(L.sph_integrate(ctx, n, arr, len(chunk)), "integrate")


def empty_like_prop(pa):
    return torch.empty(pa.get_number_of_particles(), dtype=torch.float64,
                       device=pa.get_device("x").device)
