"""Learned momentum closure: a per-particle network in place of the
momentum pair loop of a fluid array on itself.

The reference has no learned part.  The closure stands in for the
``SPHPressureGradient`` (sph/funcs/pressure_funcs.pyx:40-91) and
``MonaghanArtificialVsicosity`` (sph/funcs/viscosity_funcs.pyx:41-124) terms
that a fluid array receives from itself; boundary forces, gravity and
position stepping stay with the plain rates kernel.

Pieces (all device work is in ``csrc/mlp.cu`` and ``csrc/pairs.cu`` behind
the ``sph_mlp_*`` C ABI):

* :class:`MomentumMLP` -- the network 192 -> 128 -> 128 -> 2 (GELU), FP32
  master parameters with BF16 copies, tensor-core forward and backward,
  Adam;
* :class:`Normalisation` -- per-channel feature standardisation and the
  target scaling ``a h / c0^2`` standardised per component;
* :class:`SampleRecorder` -- hooks a solver's rates stage and stores
  (features, target) pairs of every evaluation: the features the network
  would see and the plain pair loop's accelerations at the same state;
* :func:`train` -- minibatch Adam on the recorded samples;
* :class:`LearnedClosure` -- hooks the rates stage and replaces the
  fluid-on-itself pressure gradient + viscosity by the network;
* :class:`GuardedRunner` -- advances a solver with the closure in windows
  of ``k`` steps, re-runs each checked window with the plain pair loop
  from the window's start and falls back to the plain result when the
  normwise density difference exceeds the tolerance.
"""
import ctypes

import numpy as np
import torch

from . import native
from .sph import gpu

NPARAM = native.MLP_NPARAM
NIN, NH, NOUT = native.MLP_NIN, native.MLP_NH, native.MLP_NOUT
NCH = native.MLP_NCH
SELF_KINDS = frozenset(("pgrad", "avisc"))


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class MomentumMLP:
    """The closure network on the GPU."""

    def __init__(self, seed=0, device="cuda"):
        self.device = torch.device(device)
        rng = np.random.default_rng(seed)
        p = np.zeros(NPARAM, np.float32)
        o = native
        p[o.MLP_OFF_W1:o.MLP_OFF_B1] = rng.uniform(-1, 1, NH * NIN) / np.sqrt(NIN)
        p[o.MLP_OFF_W2:o.MLP_OFF_B2] = rng.uniform(-1, 1, NH * NH) / np.sqrt(NH)
        p[o.MLP_OFF_W3:o.MLP_OFF_B3] = rng.uniform(-1, 1, NOUT * NH) / np.sqrt(NH)
        self.params = torch.as_tensor(p, device=self.device)
        self.w1 = torch.empty(NH * NIN, dtype=torch.bfloat16, device=self.device)
        self.w2 = torch.empty(NH * NH, dtype=torch.bfloat16, device=self.device)
        self.w2t = torch.empty(NH * NH, dtype=torch.bfloat16, device=self.device)
        self.w3 = torch.empty(NOUT * NH, dtype=torch.bfloat16, device=self.device)
        self.m = torch.zeros(NPARAM, dtype=torch.float32, device=self.device)
        self.v = torch.zeros(NPARAM, dtype=torch.float32, device=self.device)
        self.grad = torch.zeros(NPARAM, dtype=torch.float32, device=self.device)
        self.loss = torch.zeros(1, dtype=torch.float32, device=self.device)
        self.err = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.adam_steps = 0
        self._scratch = None
        self._model = native.MlpModel(self.params.data_ptr(), self.w1.data_ptr(),
                                      self.w2.data_ptr(), self.w2t.data_ptr(),
                                      self.w3.data_ptr())
        self.sync()

    # -- parameters -------------------------------------------------------------
    def sync(self):
        """Rewrite the BF16 copies from the FP32 parameters."""
        native.check(native.lib().sph_mlp_sync(ctypes.byref(self._model), _stream()), "mlp sync")

    def set_params(self, values):
        self.params.copy_(torch.as_tensor(np.asarray(values, np.float32)))
        self.sync()

    def state(self):
        return {"params": self.params.cpu().numpy().copy()}

    # -- forward / backward -----------------------------------------------------
    def forward(self, x, save=False):
        """``y [n, 2]`` for BF16 features ``x [n, 192]``; with ``save`` also
        the cache the backward pass reads."""
        if x.dtype != torch.bfloat16 or x.dim() != 2 or x.shape[1] != NIN or not x.is_contiguous():
            raise ValueError("features must be a contiguous bfloat16 [n, 192] tensor")
        n = x.shape[0]
        y = torch.empty((n, NOUT), dtype=torch.float32, device=self.device)
        cache = None
        if save:
            cache = dict(z1=torch.empty((n, NH), dtype=torch.float32, device=self.device),
                         z2=torch.empty((n, NH), dtype=torch.float32, device=self.device),
                         h1=torch.empty((n, NH), dtype=torch.bfloat16, device=self.device),
                         h2=torch.empty((n, NH), dtype=torch.bfloat16, device=self.device))
        c = cache or {}
        native.check(native.lib().sph_mlp_forward(
            ctypes.byref(self._model), _ptr(x), n, _ptr(y), _ptr(c.get("z1")), _ptr(c.get("z2")),
            _ptr(c.get("h1")), _ptr(c.get("h2")), _ptr(self.err), _stream()), "mlp forward")
        return (y, cache) if save else y

    def backward(self, x, cache, y, target, inv_count=None):
        """Gradient of ``0.5 * inv_count * sum (y - target)^2`` into
        ``self.grad`` and the loss into ``self.loss`` (device)."""
        n = x.shape[0]
        if inv_count is None:
            inv_count = 1.0 / n
        need = ctypes.c_int64()
        native.check(native.lib().sph_mlp_backward_scratch(n, ctypes.byref(need)), "scratch")
        if self._scratch is None or self._scratch.numel() < need.value:
            self._scratch = torch.empty(need.value, dtype=torch.float32, device=self.device)
        target = target.contiguous()
        native.check(native.lib().sph_mlp_backward(
            ctypes.byref(self._model), _ptr(x), _ptr(cache["h1"]), _ptr(cache["h2"]),
            _ptr(cache["z1"]), _ptr(cache["z2"]), _ptr(y), _ptr(target), n, float(inv_count),
            _ptr(self.grad), _ptr(self.loss), _ptr(self._scratch), _ptr(self.err), _stream()),
            "mlp backward")
        return self.grad, self.loss

    def adam(self, lr, beta1=0.9, beta2=0.999, eps=1e-8):
        self.adam_steps += 1
        native.check(native.lib().sph_mlp_adam(
            ctypes.byref(self._model), _ptr(self.grad), _ptr(self.m), _ptr(self.v), lr, beta1,
            beta2, eps, self.adam_steps, _stream()), "mlp adam")

    def check(self):
        if int(self.err.item()) & native.SPH_EFLAG_TIMEOUT:
            self.err.zero_()
            raise RuntimeError("tensor-core wait timed out in the network kernels")


class Normalisation:
    """Feature and target scaling of the closure.

    Features: per channel ``(raw - mean) * inv_std``.  Targets: ``a h / c0^2``
    per component, then ``(value - mean) / std``.
    """

    def __init__(self, c0, feat_mean=None, feat_std=None, targ_mean=None, targ_std=None):
        self.c0 = float(c0)
        self.feat_mean = np.zeros(NCH) if feat_mean is None else np.asarray(feat_mean, float)
        self.feat_std = np.ones(NCH) if feat_std is None else np.asarray(feat_std, float)
        self.targ_mean = np.zeros(2) if targ_mean is None else np.asarray(targ_mean, float)
        self.targ_std = np.ones(2) if targ_std is None else np.asarray(targ_std, float)

    def feature_params(self, identity=False):
        p = native.MlpFeatureParams()
        p.c0 = self.c0
        for c in range(NCH):
            p.mean[c] = 0.0 if identity else float(self.feat_mean[c])
            p.inv_std[c] = 1.0 if identity else float(1.0 / self.feat_std[c])
        return p


def _self_term(stage):
    for t in stage.terms:
        if t["src"] is stage.dest and SELF_KINDS <= set(t["kinds"]):
            return t
    raise NotImplementedError("the rates stage of %s has no pressure-gradient + viscosity "
                              "term from itself" % stage.dest.name)


def _fluid_stage(integrator, dest):
    from .solver.integrator import RatesStage
    for st in integrator.stages:
        if isinstance(st, RatesStage) and st.dest is dest:
            return st
    raise ValueError("no rates stage for array %s" % dest.name)


def features(cm, dest, norm, out=None, raw=False):
    """Feature rows of ``dest`` on itself from the current sorted state:
    BF16 [n, 192] (standardised), or FP32 raw values with ``raw``."""
    n = dest.get_number_of_particles()
    if out is None:
        out = torch.empty((n, NIN), dtype=torch.float32 if raw else torch.bfloat16,
                          device=dest.get_device("x").device)
    prm = norm.feature_params(identity=raw)
    cm.ensure_current()
    slot = cm.slot(dest)
    native.check(native.lib().sph_mlp_features(
        cm.context(), slot, slot, ctypes.byref(prm), None if raw else _ptr(out),
        _ptr(out) if raw else None), "features")
    return out


class SampleRecorder:
    """Record (features, target) pairs from a running plain solver.

    Attached to the rates stage of ``dest``: at every ``every``-th
    evaluation it stores the raw FP32 feature rows and the accelerations of
    the fluid-on-itself pressure gradient + viscosity at the same state
    (one extra rates launch into scratch arrays) as ``a h / c0^2``, up to
    ``capacity`` samples.  :meth:`finish` derives the normalisation from
    everything recorded and returns the standardised BF16 samples.
    """

    def __init__(self, integrator, dest, c0, capacity, every=1):
        self.stage = _fluid_stage(integrator, dest)
        self.term = _self_term(self.stage)
        self.dest = dest
        self.every = every
        self.calls = 0
        self.capacity = int(capacity)
        self.c0 = float(c0)
        self.norm = None
        dev = dest.get_device("x").device
        self.raw = torch.empty((self.capacity, NIN), dtype=torch.float32, device=dev)
        self.t = torch.empty((self.capacity, NOUT), dtype=torch.float32, device=dev)
        self.count = 0
        self.stage.hooks.append(self)

    def detach(self):
        if self in self.stage.hooks:
            self.stage.hooks.remove(self)

    @property
    def full(self):
        return self.count >= self.capacity

    def _accels(self, integ):
        cm = integ.particles.cell_manager
        n = self.dest.get_number_of_particles()
        dev = self.dest.get_device("x").device
        ax = torch.zeros(n, dtype=torch.float64, device=dev)
        ay = torch.zeros(n, dtype=torch.float64, device=dev)
        az = torch.zeros(n, dtype=torch.float64, device=dev)
        term = dict(self.term)
        term["kinds"] = set(SELF_KINDS)
        gpu.rates(cm, self.dest, [term], self.stage.dim, acc=(ax, ay, az), pos=(),
                  accumulate=False)
        return ax, ay

    # RatesStage hook -----------------------------------------------------------
    def before_rates(self, integ, stage, terms):
        return terms

    def after_rates(self, integ, stage, acc):
        self.calls += 1
        if self.full or (self.calls - 1) % self.every:
            return
        cm = integ.particles.cell_manager
        ax, ay = self._accels(integ)
        n = self.dest.get_number_of_particles()
        k = min(n, self.capacity - self.count)
        ident = Normalisation(self.c0)
        fx = features(cm, self.dest, ident, raw=True)
        tt = torch.empty((n, NOUT), dtype=torch.float32, device=fx.device)
        zero = (ctypes.c_double * 2)(0.0, 0.0)
        one = (ctypes.c_double * 2)(1.0, 1.0)
        native.check(native.lib().sph_mlp_targets(
            n, _ptr(ax), _ptr(ay), _ptr(self.dest.get_device("h")), self.c0, zero, one, _ptr(tt),
            _stream()), "targets")
        self.raw[self.count:self.count + k].copy_(fx[:k])
        self.t[self.count:self.count + k].copy_(tt[:k])
        self.count += k

    def finish(self):
        """(x BF16 [count, 192], t FP32 [count, 2], Normalisation)."""
        return standardise(self.raw[:self.count], self.t[:self.count], self.c0)


def standardise(raw, t, c0, chunk=1 << 20):
    """Normalisation from raw FP32 features (padding rows: zero density
    channel) and raw targets, and the standardised BF16 / FP32 samples."""
    n = raw.shape[0]
    rows = raw.view(n, -1, NCH)
    s1 = torch.zeros(NCH, dtype=torch.float64, device=raw.device)
    s2 = torch.zeros(NCH, dtype=torch.float64, device=raw.device)
    cnt = 0
    for a in range(0, n, chunk):
        r = rows[a:a + chunk].reshape(-1, NCH)
        r = r[r[:, 4] != 0].double()
        s1 += r.sum(0)
        s2 += (r * r).sum(0)
        cnt += r.shape[0]
    fm = (s1 / max(cnt, 1)).cpu().numpy()
    fs = np.sqrt(np.maximum((s2 / max(cnt, 1)).cpu().numpy() - fm * fm, 0.0))
    fs[fs < 1e-12 * np.maximum(np.abs(fm), 1.0)] = 1.0
    td = t.double()
    tm = td.mean(0).cpu().numpy()
    ts = td.std(0).cpu().numpy()
    ts[ts < 1e-30] = 1.0
    norm = Normalisation(c0, fm, fs, tm, ts)
    x = torch.empty((n, NIN), dtype=torch.bfloat16, device=raw.device)
    m = torch.as_tensor(fm, dtype=torch.float32, device=raw.device)
    inv = torch.as_tensor(1.0 / fs, dtype=torch.float32, device=raw.device)
    for a in range(0, n, chunk):
        r = rows[a:a + chunk]
        present = (r[..., 4] != 0).unsqueeze(-1)
        x[a:a + chunk] = torch.where(present, (r - m) * inv, 0.0).reshape(-1, NIN).to(torch.bfloat16)
    tn = ((td - torch.as_tensor(tm, device=t.device)) /
          torch.as_tensor(ts, device=t.device)).float().contiguous()
    return x, tn, norm


def train(model, x, t, epochs=10, batch=8192, lr=1e-3, lr_final=1e-5, seed=0, log=None):
    """Minibatch Adam on (x, t) with a cosine learning-rate decay; the
    samples are reshuffled every epoch.  Returns the mean loss per epoch."""
    n = x.shape[0]
    g = torch.Generator(device=x.device)
    g.manual_seed(seed)
    nb = max(1, n // batch)
    total = epochs * nb
    it = 0
    losses = []
    acc = torch.zeros(1, dtype=torch.float32, device=x.device)
    for ep in range(epochs):
        perm = torch.randperm(n, generator=g, device=x.device)
        xs = x[perm]
        ts = t[perm]
        acc.zero_()
        for b in range(nb):
            xb = xs[b * batch:(b + 1) * batch]
            tb = ts[b * batch:(b + 1) * batch]
            y, cache = model.forward(xb, save=True)
            model.backward(xb, cache, y, tb)
            frac = it / max(1, total - 1)
            cur = lr_final + 0.5 * (lr - lr_final) * (1 + np.cos(np.pi * frac))
            model.adam(float(cur))
            acc += model.loss
            it += 1
        model.check()
        losses.append(float(acc.item()) / nb)
        if log:
            log("epoch %d loss %.6g" % (ep, losses[-1]))
    return losses


class LearnedClosure:
    """Replace the fluid-on-itself pressure gradient + viscosity of ``dest``
    by the network (hooked into the integrator's rates stage)."""

    def __init__(self, integrator, dest, model, norm):
        self.stage = _fluid_stage(integrator, dest)
        self.term = _self_term(self.stage)
        self.dest = dest
        self.model = model
        self.norm = norm
        self.active = True
        rest = set(self.term["kinds"]) - SELF_KINDS
        self.reduced = []
        for t in self.stage.terms:
            if t is self.term:
                if rest:
                    r = dict(t)
                    r["kinds"] = rest
                    self.reduced.append(r)
            else:
                self.reduced.append(t)
        self._y = None
        self.stage.hooks.append(self)

    def detach(self):
        if self in self.stage.hooks:
            self.stage.hooks.remove(self)

    def before_rates(self, integ, stage, terms):
        if not self.active:
            return terms
        cm = integ.particles.cell_manager
        x = features(cm, self.dest, self.norm)
        self._y = self.model.forward(x)
        return self.reduced

    def after_rates(self, integ, stage, acc):
        if not self.active or self._y is None:
            return
        cm = integ.particles.cell_manager
        nm = self.norm
        scale = (ctypes.c_double * 2)(*nm.targ_std)
        mean = (ctypes.c_double * 2)(*nm.targ_mean)
        ptrs = (ctypes.c_void_p * 3)(*[None if a is None else a.data_ptr() for a in acc])
        native.check(native.lib().sph_mlp_apply(
            cm.context(), cm.slot(self.dest), _ptr(self._y), nm.c0, scale, mean, ptrs, 1),
            "mlp apply")
        self._y = None


STATE_PROPS = ("x", "y", "z", "u", "v", "w", "rho", "p", "cs")


class GuardedRunner:
    """Advance a solver with a learned closure in windows of ``k`` steps.

    Every ``check_every``-th window is re-run from its start with the plain
    pair loop.  The decision uses the normwise density difference between
    the two ends, ``max|rho_s - rho_p| / max|rho_p|`` (the metric of every
    parity check of the pair passes): above ``tol`` the plain result is kept
    and the closure stays off for ``cooldown`` windows, otherwise the
    surrogate result is kept.  The per-particle maximum relative difference
    is recorded beside it; at a free surface a few particles of near-zero
    density make it large even between two plain runs whose summation
    orders differ, so it is reported and not used to decide.
    """

    def __init__(self, solver, particles, closure, k=10, tol=1e-3, check_every=1, cooldown=4):
        self.integ = solver.integrator
        # a re-run window must repeat the run it checks: no skin changes
        self.integ.skin_frozen = True
        self.particles = particles
        self.closure = closure
        self.k = int(k)
        self.tol = float(tol)
        self.check_every = int(check_every)
        self.cooldown = int(cooldown)
        self.windows = 0
        self.off = 0
        self.fallbacks = 0
        self.checks = 0
        self.kept = 0                   # checked surrogate windows kept
        self.max_err = 0.0              # normwise, over the checked windows
        self.max_err_maxrel = 0.0       # per-particle maximum relative
        self.errors = []                # normwise error of every check

    def _save(self):
        return [{p: pa.get_device(p).clone() for p in STATE_PROPS if pa.has_array(p)}
                for pa in self.particles.arrays]

    def _restore(self, snap):
        for pa, s in zip(self.particles.arrays, snap):
            pa.set(**s)
        # a full build from the restored state: the replay then depends on
        # the state alone, exactly as the run it repeats
        self.particles.cell_manager.rebuild(check_jump=False)

    def _steps(self, dt, n):
        for _ in range(n):
            self.integ.integrate(dt)

    def window(self, dt):
        """One window of ``k`` steps."""
        self.windows += 1
        if self.off > 0:
            self.off -= 1
            self.closure.active = False
            self._steps(dt, self.k)
            return
        check = (self.windows - 1) % self.check_every == 0
        self.particles.cell_manager.rebuild()
        start = self._save()
        self.closure.active = True
        try:
            self._steps(dt, self.k)
            failed = False
        except RuntimeError:
            # the surrogate moved a particle by more than a cell: a failed window
            failed = True
        if not check and not failed:
            return
        self.checks += 1
        surr = None if failed else self._save()
        self._restore(start)
        self.closure.active = False
        self._steps(dt, self.k)
        dest = self.closure.dest
        i = self.particles.arrays.index(dest)
        rp = dest.get_device("rho")
        if failed:
            err = rel = float("inf")
        else:
            d = (surr[i]["rho"] - rp).abs()
            err = float((d.max() / rp.abs().max()).item())
            rel = float((d / rp.abs()).max().item())
        self.errors.append(err)
        self.max_err = max(self.max_err, err)
        self.max_err_maxrel = max(self.max_err_maxrel, rel)
        if err > self.tol:
            self.fallbacks += 1
            self.off = self.cooldown
        else:
            self.kept += 1
            self._restore(surr)
        self.closure.active = True

    def stats(self):
        """Windows run, checked, kept and fallen back, with the errors."""
        errs = sorted(self.errors)
        return {"windows": self.windows, "checks": self.checks, "kept": self.kept,
                "fallbacks": self.fallbacks,
                "fallback_rate": self.fallbacks / self.checks if self.checks else None,
                "min_normwise_density_error": errs[0] if errs else None,
                "median_normwise_density_error": errs[len(errs) // 2] if errs else None,
                "max_normwise_density_error": self.max_err,
                "max_relative_density_error": self.max_err_maxrel}


def dam_break_samples(api, aspects, dx=0.01, dt=1e-4, steps=2000, every=40, capacity=None,
                      height=2.0, log=None):
    """Record closure samples from plain dam-break runs, one per column
    aspect ratio (width / height): the fluid-on-itself pressure gradient +
    viscosity of every ``every``-th evaluation.  Returns the raw FP32
    features, raw targets and c0 (samples of all runs concatenated)."""
    from . import workloads as W
    c0 = W.dam_break_c0(height=height)
    raws, targs = [], []
    left = capacity
    for a in aspects:
        fluid, wall = W.dam_break(dx=dx, column=(a * height, height))
        s, particles = W.setup_dam_break(api, fluid, wall, dx, c0)
        fl = particles.arrays[0]
        n = fl.get_number_of_particles()
        cap = (2 * steps // every + 1) * n
        if left is not None:
            cap = min(cap, left // max(1, len(aspects) - len(raws)))
        rec = SampleRecorder(s.integrator, fl, c0, capacity=cap, every=every)
        for _ in range(steps):
            s.integrator.integrate(dt)
            if rec.full:
                break
        rec.detach()
        raws.append(rec.raw[:rec.count])
        targs.append(rec.t[:rec.count])
        if left is not None:
            left -= rec.count
        if log:
            log("aspect %.3f: %d fluid particles, %d samples" % (a, n, rec.count))
        del s, particles
    return torch.cat(raws), torch.cat(targs), c0
