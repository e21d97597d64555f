"""Euler, RK2, RK4, predictor-corrector and leap-frog integrators driving
the GPU stages.

Reference: solver/integrator.py.  The reference evaluates its calcs one by
one (``eval`` :432-470), storing every integrating calc's result in its own
``_k<n>_<prop><i><j>`` array, then steps the properties with NumPy
(``step`` :472-514, ``final_step`` of Euler :535-553, RK2 :597-619, RK4
:669-692, PredictorCorrector :751-765, LeapFrog :874-891).  Here
``setup_integrator`` compiles the calc list into stages:

* ``DensityStage``  -- SPHRho over all its sources, fused with an
  immediately following TaitEquation on the same destination (the first
  pair pass after a neighbour build also writes the neighbour lists);
* ``TaitStage``     -- a TaitEquation on its own (e.g. before SPHRho);
* ``RatesStage``    -- a maximal run of consecutive integrating calcs on one
  destination (pressure gradient, artificial viscosity, boundary force,
  XSPH, gravity, position stepping) as ONE rates-kernel launch writing the
  summed rate of each integrated property.

Integrating calcs only write rates, never state, so merging a consecutive
run of them changes nothing but the order of the FP64 additions (the
reference adds each calc's ``k*dt`` in turn).  The state update is one FP64
kernel per array with the rounding of the reference's NumPy expressions.
"""
import ctypes
import logging

import torch

from ..sph import gpu
from ..sph.sph_calc import RATE_KINDS, _kind_of, _term

logger = logging.getLogger()

VEL = ("u", "v", "w")
POS = ("x", "y", "z")
RHO = ("rho",)
VEL_KINDS = ("pgrad", "avisc", "bforce", "gravity", "momentum")
POS_KINDS = ("xsph", "step")
RHO_KINDS = ("drho",)


class DensityStage:
    def __init__(self, calc, tait=None):
        self.calc = calc
        self.tait = tait
        self.dest = calc.dest

    def run(self, integ, kname):
        c = self.calc
        cm = integ.particles.cell_manager
        rho = self.dest.get_device(c.updates[0])
        if self.tait is not None:
            t = self.tait.funcs[0]
            p = self.dest.get_device(self.tait.updates[0])
            cs = self.dest.get_device(self.tait.updates[1])
            gpu.density(cm, self.dest, c.sources, c.kernel.dim, rho, (t.co, t.ro, t.gamma), p, cs)
            names = [c.updates[0]] + list(self.tait.updates)
            own = names == ["rho", "p", "cs"]
        else:
            gpu.density(cm, self.dest, c.sources, c.kernel.dim, rho)
            names = [c.updates[0]]
            own = names == ["rho"]
        gpu.note_written(cm, self.dest, names, consistent=own)


class TaitStage:
    def __init__(self, calc):
        self.calc = calc
        self.dest = calc.dest

    def run(self, integ, kname):
        c = self.calc
        f = c.funcs[0]
        cm = integ.particles.cell_manager
        gpu.tait(cm, self.dest, f.co, f.ro, f.gamma, self.dest.get_device(c.updates[0]),
                 self.dest.get_device(c.updates[1]))
        gpu.note_written(cm, self.dest, c.updates)


class CalcStage:
    """A non-integrating calc evaluated on its own (``calc.sph(*updates)``)."""

    def __init__(self, calc):
        self.calc = calc
        self.dest = calc.dest

    def run(self, integ, kname):
        self.calc.sph(*self.calc.updates)


class RatesStage:
    def __init__(self, calcs):
        self.calcs = calcs
        self.dest = calcs[0].dest
        self.terms = []
        self.gravity = None
        self.add_velocity = False
        self.props = []
        # objects with before_rates(integ, stage, terms) -> terms and
        # after_rates(integ, stage, acc) (learned closure, sample recorder)
        self.hooks = []
        dim = None
        for c in calcs:
            kind = _kind_of(c.funcs[0])
            if kind not in RATE_KINDS + ("gravity", "step"):
                raise NotImplementedError("%s cannot be integrated on the GPU" % kind)
            allowed = VEL if kind in VEL_KINDS else (RHO if kind in RHO_KINDS else POS)
            if list(c.updates) != list(allowed[:len(c.updates)]):
                raise NotImplementedError(
                    "calc %s updates %s; the GPU integrator needs a prefix of %s"
                    % (c.id, c.updates, allowed))
            for p in c.updates:
                if p not in self.props:
                    self.props.append(p)
            if kind in RATE_KINDS:
                dim = c.kernel.dim if dim is None else dim
                if c.kernel.dim != dim:
                    raise NotImplementedError("mixed kernel dimensions in one rates stage")
                for f in c.funcs:
                    self._add_term(_term(f, kind))
            elif kind == "gravity":
                f = c.funcs[0]
                g = self.gravity or (0.0, 0.0, 0.0)
                self.gravity = (g[0] + f.gx, g[1] + f.gy, g[2] + f.gz)
            else:
                if self.add_velocity:
                    raise NotImplementedError("two position-stepping calcs on one array")
                self.add_velocity = True
        self.dim = dim or 3

    def _add_term(self, t):
        # merge different kinds on the same source into one traversal (only
        # when their term flags are disjoint: MomentumEquation is PGrad + AV)
        def flags(kinds):
            f = 0
            for k in kinds:
                f |= gpu.RATE_TERM[k]
            return f
        for e in self.terms:
            if e["src"] is t["src"] and not (flags(e["kinds"]) & flags(t["kinds"])):
                e["kinds"] = e["kinds"] | t["kinds"]
                for k, v in t.items():
                    if k not in ("src", "kinds"):
                        e[k] = v
                return
        self.terms.append(dict(t))

    def run(self, integ, kname):
        cm = integ.particles.cell_manager
        rate = integ.rate_arrays(self.dest, kname)
        written = integ._written.setdefault(id(self.dest), set())
        fresh = [p for p in self.props if p not in written]
        if fresh and len(fresh) != len(self.props):
            if getattr(cm, "recording", False):
                raise RuntimeError("a partly written rate array cannot be recorded")
            for p in fresh:
                rate[p].zero_()
            fresh = []
        accumulate = not fresh
        acc = [rate.get(p) if p in self.props else None for p in VEL]
        pos = [rate.get(p) if p in self.props else None for p in POS]
        drho = rate.get("rho") if "rho" in self.props else None
        terms = self.terms
        for hk in self.hooks:
            terms = hk.before_rates(integ, self, terms)
        if terms or self.gravity or self.add_velocity or (self.hooks and not accumulate):
            gpu.rates(cm, self.dest, terms, self.dim, acc=acc, pos=pos,
                      accumulate=accumulate, gravity=self.gravity,
                      add_velocity=self.add_velocity, drho=drho)
        for hk in self.hooks:
            hk.after_rates(integ, self, acc)
        written.update(self.props)


class Integrator:
    """solver/integrator.py:9-519."""

    def __init__(self, particles=None, calcs=None, pcalcs=None):
        self.particles = particles
        self.calcs = list(calcs or [])
        self.icalcs = []
        self.pcalcs = []
        self.nsteps = 1
        self.cstep = 1
        self.initial_props = {}
        self.k_props = {}
        self.setup_done = False
        self.rupdate_list = []
        self.stages = []
        self._rates = {}
        self._written = {}
        # array versions right after a final update that left X0 = X
        self._x0_versions = None
        # when a list, CUDA events (name, start, end) are recorded around
        # every stage and neighbour build on the current stream
        self.stage_events = None
        self._replay = None
        self._steps_done = 0
        self._saved_count = 0

    def set_rupdate_list(self):
        self.rupdate_list = [[] for _ in self.particles.arrays]

    def setup_integrator(self):
        """integrator.py:229-337 bookkeeping plus the stage plan."""
        self.arrays = self.particles.arrays
        cm = getattr(self.particles, "cell_manager", None)
        if cm is not None:
            # every update of a step is followed by its pair passes
            cm.set_deferred_check(True)
        calcs = self.calcs
        self.pcalcs = [c for c in calcs if c.tag == "position"]
        self.ncalcs = [c for c in calcs if not c.tag == "position"]
        self.icalcs = [c for c in calcs if not c.tag == "position" and c.integrates]
        self.initial_props = {}
        self.k_props = {}
        for i, calc in enumerate(calcs):
            pa = self.arrays[calc.dnum]
            self.initial_props[calc.id] = []
            self.k_props[calc.id] = {}
            for j, prop in enumerate(calc.updates):
                prop_initial = "_" + prop + "_0"
                if calc.integrates:
                    pa.add_property({"name": prop_initial})
                    if prop_initial not in calc.initial_props:
                        calc.initial_props.append(prop_initial)
                self.initial_props[calc.id].append(prop_initial)
                for l in range(self.nsteps):
                    k_num = "k" + str(l + 1)
                    if calc.integrates:
                        self.k_props[calc.id].setdefault(k_num, [])
                        k_name = "_" + k_num + "_" + prop + str(i) + str(j)
                        calc.dst_writes.setdefault(k_num, [])
                        if k_name not in calc.dst_writes[k_num]:
                            calc.dst_writes[k_num].append(k_name)
                        self.k_props[calc.id][k_num].append(k_name)
        self._plans = {}
        self._x0_versions = None
        self.stages = self._make_plans()
        self._integrated = {}
        for st in self.stages:
            if isinstance(st, RatesStage):
                lst = self._integrated.setdefault(id(st.dest), (st.dest, []))[1]
                for p in st.props:
                    if p not in lst:
                        lst.append(p)
        for dest, props in self._integrated.values():
            for l in range(self.nsteps):
                for p in props:
                    dest.add_property({"name": "_rate%d_%s" % (l + 1, p)})
        self.set_rupdate_list()
        self.setup_done = True

    def _make_plans(self):
        """The stage list of one step (the learned closure hooks its stages)."""
        return self._plan(self.calcs)

    def _stages_for(self, calcs):
        if calcs is None or calcs is self.calcs:
            return self.stages
        key = tuple(id(c) for c in calcs)
        if key not in self._plans:
            self._plans[key] = self._plan(list(calcs))
        return self._plans[key]

    @staticmethod
    def _plan(calcs):
        stages = []
        i = 0
        while i < len(calcs):
            c = calcs[i]
            kind = _kind_of(c.funcs[0])
            if not c.integrates:
                if kind == "rho":
                    nxt = calcs[i + 1] if i + 1 < len(calcs) else None
                    if (nxt is not None and not nxt.integrates and nxt.dest is c.dest
                            and _kind_of(nxt.funcs[0]) == "tait" and c.updates == ["rho"]):
                        stages.append(DensityStage(c, nxt))
                        i += 2
                        continue
                    stages.append(DensityStage(c))
                elif kind == "tait":
                    stages.append(TaitStage(c))
                else:
                    stages.append(CalcStage(c))
                i += 1
                continue
            run = [c]
            j = i + 1
            while j < len(calcs) and calcs[j].integrates and calcs[j].dest is c.dest:
                run.append(calcs[j])
                j += 1
            stages.append(RatesStage(run))
            i = j
        return stages

    def rate_arrays(self, dest, kname):
        return {p: dest.get_device("_rate%s_%s" % (kname[1:], p))
                for p in self._integrated[id(dest)][1]}

    # -- the reference's step building blocks ------------------------------------
    def eval(self, calcs=None):
        """Evaluate the stages of ``calcs`` (default: all) for the current
        ``cstep`` (integrator.py:432-470)."""
        kname = "k" + str(self.cstep)
        self._written = {}
        for st in self._stages_for(calcs):
            if self.stage_events is None:
                st.run(self, kname)
            else:
                self._timed(type(st).__name__, st.run, self, kname)

    def _timed(self, name, fn, *args):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        fn(*args)
        b.record()
        self.stage_events.append((name, a, b))

    def _update_particles(self):
        if self.stage_events is None:
            self.particles.update()
        else:
            self._timed("NNPSBuild", self.particles.update)

    def _props_of(self, calcs):
        """{id(dest): set of integrated properties} of the integrating calcs."""
        out = {}
        for c in calcs:
            if c.integrates:
                out.setdefault(id(c.dest), set()).update(c.updates)
        return out

    def _lines(self, mode, dt, level=1, calcs=None):
        """Integrator lines (``gpu.axpy`` tuples) of every integrated property
        (of ``calcs`` only, when given), grouped per destination array."""
        only = None if calcs is None else self._props_of(calcs)
        out = []
        for dest, props in self._integrated.values():
            if only is not None:
                props = [p for p in props if p in only.get(id(dest), ())]
            if not props:
                continue
            n = dest.get_number_of_particles()
            lines = []
            for p in props:
                cur = dest.get_device(p)
                init = dest.get_device("_" + p + "_0")

                def r(l, p=p):
                    return dest.get_device("_rate%d_%s" % (l, p))

                if mode == "copy":        # set_initial_arrays
                    lines.append((init, None, cur, None, None, 0.0, 2))
                elif mode == "reset":     # reset_current_arrays
                    lines.append((cur, None, init, None, None, 0.0, 2))
                elif mode == "euler":     # X0 + k1 dt, X0 <- X
                    lines.append((cur, init, init, r(1), None, dt, 1))
                elif mode == "predict":   # reset + step: X0 + k_level dt
                    lines.append((cur, None, init, r(level), None, dt, 1))
                elif mode == "rk2":       # X0 + dt/2 (k1 + k2), X0 <- X
                    lines.append((cur, init, init, r(1), r(2), 0.5 * dt, 0))
                elif mode == "rk4":       # X0 + dt/6 (k1 + 2k2 + 2k3 + k4), X0 <- X
                    lines.append((cur, init, init, r(1), r(2), dt / 6.0, 5, r(3), r(4)))
                elif mode == "pc":        # 2X - X0, X0 <- X
                    lines.append((cur, init, cur, init, None, 0.0, 3))
                elif mode == "leapfrog":  # X + dt/2 (k2 - k1)
                    lines.append((cur, None, cur, r(1), r(2), 0.5 * dt, 4))
                else:
                    raise ValueError(mode)
            out.append((dest, n, props, lines))
        return out

    def _apply(self, mode, dt=0.0, level=1, calcs=None):
        cm = self.particles.cell_manager
        for dest, n, props, lines in self._lines(mode, dt, level, calcs):
            gpu.axpy(cm, n, lines)
            if mode != "copy":
                gpu.note_written(cm, dest, props)
                if any(p in POS for p in props):
                    dest.set_dirty(True)

    def set_initial_arrays(self):
        """X0 = X for every integrated property (integrator.py:339-367).
        Skipped when the last step's final update already left X0 = X and
        no array changed since."""
        if self._x0_versions is not None and all(
                self._x0_versions.get(id(dest)) == dest.version
                for dest, _ in self._integrated.values()):
            return
        self._apply("copy")

    def _saved_initial(self):
        """The final update just wrote X0 = X (its lines save the result)."""
        self._x0_versions = {id(dest): dest.version for dest, _ in self._integrated.values()}
        self._saved_count += 1

    def reset_current_arrays(self, calcs=None):
        self._apply("reset", calcs=calcs)

    def step(self, calcs=None, dt=0.0):
        """The reference's reset_current_arrays + step: X = X0 + dt k_cstep
        for the integrating calcs of ``calcs`` (default: all)."""
        self._apply("predict", dt, level=self.cstep, calcs=calcs)
        self.cstep += 1

    def do_step(self, calcs=None, dt=0.0):
        """integrator.py:380-411: evaluate, then step from the initial arrays."""
        self.eval(calcs)
        self.step(calcs, dt)

    def _integrate(self, dt):
        raise NotImplementedError

    def integrate(self, dt):
        """One time step.  From the second step on, the step's calls of the
        C ABI are recorded once into a step program (``sph_step_*``), which
        then runs each later step as one CUDA graph while the arrays, dt
        and the stage plan stay as they were (any change, or the learned
        closure's hooks, or per-stage timing, runs the step call by call
        and records afresh).  Results are those of the calls run one by
        one."""
        if not self.setup_done:
            self.setup_integrator()
        rp = self._replay
        if rp is not None:
            if rp.usable(self, dt):
                rp.run()
                self._steps_done += 1
                self._adapt_skin()
                return
            self._drop_replay()
        if self._steps_done >= 1 and self._may_record():
            rp = StepReplay.record(self, dt)
            if rp is not None:
                self._replay = rp
                rp.run()
                self._steps_done += 1
                self._adapt_skin()
                return
        self._integrate(dt)
        self._steps_done += 1
        self._adapt_skin()

    def _adapt_skin(self):
        """Grow the neighbour-list skin of a small simulation whose lists go
        stale within a few steps (``tuning.skin_growth``): every SKIN_WINDOW
        steps, while the window had more than one full build per four steps,
        the skin doubles (up to SKIN_MAX)."""
        from .. import tuning
        if getattr(self, "skin_frozen", False) or not torch.cuda.is_available():
            return
        n = sum(pa.get_number_of_particles() for pa in self.particles.arrays)
        rule = tuning.skin_growth(n)
        if rule is None:
            return
        window, most, factor, ceiling = rule
        if self._steps_done % window != 0:
            return
        cm = getattr(self.particles, "cell_manager", None)
        if cm is None or cm._ctx is None:
            return
        # full builds only: steps replayed as graphs and steps run call by
        # call count them alike (not so the light refreshes a stale one
        # replaces), so both take the same decisions
        full = cm.build_stats()[0]
        last = getattr(self, "_skin_window", None)
        self._skin_window = full
        if last is None:
            return
        skin = cm.list_skin()
        if full - last > most and 0.0 < skin < ceiling:
            cm.set_skin(min(ceiling, factor * skin))
            # the next window starts after the build the new skin forced
            self._skin_window = cm.build_stats()[0]

    def _may_record(self):
        from ..tuning import step_graphs
        n = sum(pa.get_number_of_particles() for pa in self.particles.arrays)
        if not step_graphs(n) or self.stage_events is not None:
            return False
        cm = getattr(self.particles, "cell_manager", None)
        if cm is None or not torch.cuda.is_available():
            return False
        return not self._unrecordable_stages()

    def _unrecordable_stages(self):
        """Whether a stage runs work a step program does not record: the
        learned closure's hooks and calcs evaluated on their own
        (SPHCalc.sph) run torch operations."""
        for st in self.stages + [s for p in self._plans.values() for s in p]:
            if isinstance(st, CalcStage) or (isinstance(st, RatesStage) and st.hooks):
                return True
        return False

    def _drop_replay(self):
        if self._replay is not None:
            self._replay.close()
            self._replay = None

    def step_stats(self):
        """Counters of the recorded step (graph replays, eager steps,
        resumed steps, captures, recorded calls, kernels per replay), or
        None."""
        return None if self._replay is None else self._replay.stats()


class EulerIntegrator(Integrator):
    """X(t+h) = X + h F(X), integrator.py:525-573."""

    def __init__(self, particles, calcs=None):
        Integrator.__init__(self, particles, calcs)
        self.nsteps = 1

    def _integrate(self, dt):
        if not self.setup_done:
            self.setup_integrator()
        self.set_initial_arrays()
        self.cstep = 1
        self.eval(self.calcs)
        self._apply("euler", dt)
        self._saved_initial()
        self._update_particles()


class RK2Integrator(Integrator):
    """X(t+h) = X + h/2 (K1 + K2), integrator.py:581-645."""

    def __init__(self, particles, calcs=None):
        Integrator.__init__(self, particles, calcs)
        self.nsteps = 2

    def _integrate(self, dt):
        if not self.setup_done:
            self.setup_integrator()
        self.set_initial_arrays()
        self.cstep = 1
        self.do_step(self.calcs, dt)
        self._update_particles()
        self.eval(self.calcs)
        self._apply("rk2", dt)
        self._saved_initial()
        self.cstep = 1
        self._update_particles()


class RK4Integrator(Integrator):
    """X(t+h) = X + h/6 (K1 + 2K2 + 2K3 + K4), integrator.py:650-730.

    K1 = F(X), K2 = F(X + h/2 K1), K3 = F(X + h/2 K2), K4 = F(X + h K3);
    four pair-loop evaluations and four neighbour builds per step."""

    def __init__(self, particles, calcs=None):
        Integrator.__init__(self, particles, calcs)
        self.nsteps = 4

    def _integrate(self, dt):
        if not self.setup_done:
            self.setup_integrator()
        self.set_initial_arrays()
        self.cstep = 1
        self.do_step(self.calcs, 0.5 * dt)
        self._update_particles()
        self.do_step(self.calcs, 0.5 * dt)
        self._update_particles()
        self.do_step(self.calcs, dt)
        self._update_particles()
        self.eval(self.calcs)
        self._apply("rk4", dt)
        self._saved_initial()
        self.cstep = 1
        self._update_particles()


class PredictorCorrectorIntegrator(Integrator):
    """integrator.py:734-796: X* = X + h/2 F(X); X** = X + h/2 F(X*);
    X(t+h) = 2 X** - X."""

    def __init__(self, particles, calcs=None):
        Integrator.__init__(self, particles, calcs)
        self.nsteps = 2

    def _integrate(self, dt):
        if not self.setup_done:
            self.setup_integrator()
        self.set_initial_arrays()
        self.cstep = 1
        self.do_step(self.calcs, 0.5 * dt)
        self._update_particles()
        self.do_step(self.calcs, 0.5 * dt)
        self._update_particles()
        self._apply("pc", dt)
        self._saved_initial()
        self._update_particles()
        self.cstep = 1


class LeapFrogIntegrator(Integrator):
    """integrator.py:802-912.

    Non-position calcs (tag != "position") and position calcs are evaluated
    separately: v* = v0 + h F0; then the position calcs see v*, x = x0 + h k_x
    and every velocity calc adds h^2/2 F0 to the first position calc's
    properties, component by component (``add_correction_for_position``);
    after a neighbour update the non-position calcs are evaluated again and
    v = v* + h/2 (F - F0) (likewise for other integrated non-position
    properties, e.g. a density rate)."""

    def __init__(self, particles, calcs=None):
        Integrator.__init__(self, particles, calcs)
        self.nsteps = 2

    def _make_plans(self):
        nst = self._plan(self.ncalcs)
        pst = self._plan(self.pcalcs)
        self._plans[tuple(id(c) for c in self.ncalcs)] = nst
        self._plans[tuple(id(c) for c in self.pcalcs)] = pst
        return nst + pst

    def _correction_lines(self, dt):
        """add_correction_for_position (integrator.py:841-872)."""
        if not self.pcalcs:
            raise IndexError("list index out of range")
        pos_calc = self.pcalcs[0]
        pos_updates = list(pos_calc.updates)
        vel_props = []
        for calc in self.icalcs:
            if calc.tag != "velocity":
                continue
            if calc.dest is not pos_calc.dest:
                raise NotImplementedError("LeapFrog position correction across two arrays")
            for j in range(len(calc.updates)):
                if j >= len(pos_updates):
                    raise IndexError("list index out of range")
                if j >= len(vel_props):
                    vel_props.append(calc.updates[j])
        dest = pos_calc.dest
        c = 0.5 * dt * dt
        lines = []
        for j, vp in enumerate(vel_props):
            x = dest.get_device(pos_updates[j])
            lines.append((x, None, x, dest.get_device("_rate1_" + vp), None, c, 1))
        return dest, lines

    def _integrate(self, dt):
        if not self.setup_done:
            self.setup_integrator()
        dest, corr = self._correction_lines(dt)
        self.set_initial_arrays()
        self.cstep = 1
        self.do_step(self.ncalcs, dt)
        self.cstep = 1
        self.do_step(self.pcalcs, dt)
        cm = self.particles.cell_manager
        if corr:
            gpu.axpy(cm, dest.get_number_of_particles(), corr)
            gpu.note_written(cm, dest, list(self.pcalcs[0].updates))
            dest.set_dirty(True)
        self._update_particles()
        self.eval(self.ncalcs)
        self._apply("leapfrog", dt, calcs=self.icalcs)
        self.cstep = 1


class StepReplay:
    """A step recorded as a step program of the C ABI and its replay
    conditions: the same dt and the same arrays (sizes and device buffers).
    Values written into the arrays between steps are taken as an eager step
    takes them: X0 = X for the integrated properties and a neighbour update
    (or snapshot refresh) of the changed arrays run before the replay."""

    def __init__(self, integ, dt, handle):
        self.integ = integ
        self.dt = dt
        self.handle = handle
        self.cm = integ.particles.cell_manager
        self.ctx = self.cm.context()
        self.signature = self._signature(integ)
        self.builds_per_step = 0

    @staticmethod
    def _arrays(integ):
        return list(integ.particles.arrays)

    @classmethod
    def _signature(cls, integ):
        sig = []
        for pa in cls._arrays(integ):
            sig.append((id(pa), pa.get_number_of_particles(),
                        tuple((k, t.data_ptr()) for k, t in sorted(pa.properties.items()))))
        return tuple(sig)

    @classmethod
    def record(cls, integ, dt):
        """Record one step (nothing runs on the device); None when a call of
        the step cannot be recorded."""
        from .. import native
        cm = integ.particles.cell_manager
        ctx = cm.context()
        L = native.lib()
        native.check(L.sph_step_begin(ctx), "sph_step_begin")
        b0 = cm._build_count
        s0 = integ._saved_count
        handle = ctypes.c_void_p()
        cm.recording = True
        try:
            integ._integrate(dt)
        except Exception:
            cm.recording = False
            L.sph_step_end(ctx, ctypes.byref(handle))
            L.sph_step_destroy(handle)
            # the recorded calls never ran: the next step updates afresh
            for pa in integ.particles.arrays:
                pa.set_dirty(True)
            cm.is_dirty = True
            integ._may_record = lambda: False
            return None
        cm.recording = False
        native.check(L.sph_step_end(ctx, ctypes.byref(handle)), "sph_step_end")
        rp = cls(integ, dt, handle)
        rp.builds_per_step = cm._build_count - b0
        # the step's final lines save X0 = X (not the leap-frog's)
        rp.saves_initial = integ._saved_count != s0
        rp.recorded = True
        return rp

    def usable(self, integ, dt):
        # hooks attached after the recording (a learned closure) change the
        # step: it runs call by call again
        return (dt == self.dt and self.cm.context().value == self.ctx.value
                and integ.stage_events is None and self._signature(integ) == self.signature
                and not integ._unrecordable_stages())

    def run(self):
        from .. import native
        integ, cm = self.integ, self.cm
        if self.recorded:
            # the step just recorded: its bookkeeping ran while recording
            self.recorded = False
        else:
            # what the eager step does first when arrays changed since the
            # last step: X0 = X, and snapshots of changed arrays
            integ.set_initial_arrays()
            cm.ensure_current()
        cm.context()   # the current stream
        native.check(native.lib().sph_step_run(self.handle, 1), "step")
        if self.saves_initial:
            integ._saved_initial()
        # locators compare the build count with their cached lists
        cm._build_count += self.builds_per_step

    def stats(self):
        from .. import native
        out = (ctypes.c_int64 * 10)()
        native.check(native.lib().sph_step_stats(self.handle, out), "sph_step_stats")
        return {"graph_steps": out[0], "eager_steps": out[1], "resumed_steps": out[2],
                "captures": out[3], "calls": out[4], "kernels_per_replay": out[5],
                "replay_device_us": out[6], "capture_attempts": out[7],
                "last_capture_failure": out[8], "graph_updates": out[9]}

    def close(self):
        from .. import native
        if self.handle:
            native.lib().sph_step_destroy(self.handle)
            self.handle = None
