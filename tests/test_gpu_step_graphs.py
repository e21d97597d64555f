"""Recorded steps replayed as CUDA graphs against the same steps run call by
call (``PYSPH_GB300_GRAPHS=0``): the replay runs the same kernels on the same
data, so trajectories agree bit for bit -- with light refreshes, with steps
whose refresh is found stale in the middle (resumed after a full build),
with values written into the arrays between steps, and with two arrays
(fluid and walls) -- and a jump is still reported as RuntimeError."""
import numpy as np
import pytest
import torch

import oracle
import pysph_gb300
from golden_util import normwise
from pysph_gb300 import workloads as W

pytestmark = pytest.mark.gpu
API = pysph_gb300.api()


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")


def _run(setup, steps, dt, graphs, monkeypatch, between=None, props=("x", "y", "z", "u", "v", "w", "rho", "p")):
    monkeypatch.setenv("PYSPH_GB300_GRAPHS", "1" if graphs else "0")
    s, particles = setup()
    pa = particles.arrays[0]
    for k in range(steps):
        if between is not None:
            between(k, pa)
        s.integrator.integrate(dt)
    out = {p: pa.get(p) for p in props if pa.has_array(p)}
    return out, s.integrator.step_stats(), particles


def _same(a, b):
    for p in a:
        np.testing.assert_array_equal(a[p], b[p], err_msg=p)


def test_cube_rk2_graph_replay_matches_eager(monkeypatch):
    _need_gpu()
    props = W.cube_lattice(32768, seed=31)
    setup = lambda: W.setup_cube(API, props)   # noqa: E731
    a, st, _ = _run(setup, 30, 1e-4, True, monkeypatch)
    b, st0, _ = _run(setup, 30, 1e-4, False, monkeypatch)
    assert st is not None and st["graph_steps"] >= 20, st
    assert st0 is None
    _same(a, b)


def test_drop_euler_graph_replay_matches_eager_and_oracle(monkeypatch):
    """2D drop (XSPH, position stepping), Euler: 60 steps."""
    _need_gpu()
    props = W.elliptical_drop(dx=0.025, c0=100.0)
    setup = lambda: W.setup_drop(API, props, c0=100.0)   # noqa: E731
    a, st, _ = _run(setup, 60, 1e-5, True, monkeypatch, props=("x", "y", "u", "v", "rho", "p"))
    b, _, _ = _run(setup, 60, 1e-5, False, monkeypatch, props=("x", "y", "u", "v", "rho", "p"))
    _same(a, b)
    # this flow moves by half the list skin within every step: every update
    # rebuilds, which the recorded step leaves to its eager calls
    print(st)
    assert st["eager_steps"] + st["graph_steps"] + st["resumed_steps"] == 59, st
    prob = oracle.Problem({"fluid": props}, oracle.drop_ops(c0=100.0), dim=2)
    for _ in range(60):
        prob.integrate_euler(1e-5)
    ref = prob.arrays["fluid"]
    for p in ("x", "y"):
        assert normwise(a[p] - props[p], ref[p] - props[p]) < 1e-4, p


def test_dam_break_two_arrays_graph_replay_matches_eager(monkeypatch):
    """Fluid and walls (boundary force from a second array), RK2."""
    _need_gpu()
    dx = 0.04
    fluid, wall = W.dam_break(dx=dx)
    c0 = W.dam_break_c0()
    setup = lambda: W.setup_dam_break(API, fluid, wall, dx, c0)   # noqa: E731
    a, st, _ = _run(setup, 40, 1e-4, True, monkeypatch, props=("x", "y", "u", "v", "rho", "p"))
    b, _, _ = _run(setup, 40, 1e-4, False, monkeypatch, props=("x", "y", "u", "v", "rho", "p"))
    _same(a, b)
    print(st)
    assert st["graph_steps"] >= 1, st


def test_stale_refresh_inside_a_replayed_step_resumes(monkeypatch):
    """Velocities large enough that particles cross half the list skin every
    few steps: light refreshes found stale inside replayed steps resume
    after a full build, and the trajectory still equals the eager one."""
    _need_gpu()
    props = W.cube_lattice(32768, seed=32, vel_std=0.5)
    setup = lambda: W.setup_cube(API, props)   # noqa: E731
    a, st, _ = _run(setup, 60, 1e-4, True, monkeypatch)
    b, _, _ = _run(setup, 60, 1e-4, False, monkeypatch)
    _same(a, b)
    print(st)
    assert st["resumed_steps"] >= 1 and st["graph_steps"] >= 1, st


def test_values_written_between_replayed_steps(monkeypatch):
    """Writing velocities and positions between steps (as the staged
    transfers do) is taken by a replayed step as by an eager one."""
    _need_gpu()
    props = W.cube_lattice(8000, seed=33)
    rng = np.random.default_rng(5)
    kicks = [rng.normal(0.0, 1e-3, 8000) for _ in range(20)]

    def between(k, pa):
        if k >= 2 and k % 3 == 0:
            u = pa.get("u")
            pa.set(u=u + kicks[k])
        if k >= 2 and k % 7 == 0:
            x = pa.get("x")
            pa.set(x=x + 1e-6)

    setup = lambda: W.setup_cube(API, props)   # noqa: E731
    a, st, _ = _run(setup, 20, 1e-4, True, monkeypatch, between=between)
    b, _, _ = _run(setup, 20, 1e-4, False, monkeypatch, between=between)
    assert st["graph_steps"] >= 10, st
    _same(a, b)


def test_jump_is_reported_from_a_replayed_step(monkeypatch):
    _need_gpu()
    monkeypatch.setenv("PYSPH_GB300_GRAPHS", "1")
    props = W.cube_lattice(8000, seed=34)
    s, particles = W.setup_cube(API, props)
    for _ in range(4):
        s.integrator.integrate(1e-4)
    assert s.integrator.step_stats()["graph_steps"] >= 1
    pa = particles.arrays[0]
    # a particle far beyond one cell in one step: the next step's first
    # refresh reports the jump
    u = pa.get("u")
    u[17] = 1e4
    pa.set(u=u)
    with pytest.raises(RuntimeError, match="more than one cell"):
        for _ in range(3):
            s.integrator.integrate(1e-4)


def test_locators_see_replayed_steps(monkeypatch):
    """Exported neighbour lists after replayed steps are those of the
    current positions."""
    _need_gpu()
    monkeypatch.setenv("PYSPH_GB300_GRAPHS", "1")
    props = W.cube_lattice(8000, seed=35, vel_std=0.1)
    s, particles = W.setup_cube(API, props)
    pa = particles.arrays[0]
    loc = particles.nnps_manager.get_neighbor_particle_locator(pa, pa, 2.0)
    loc.neighbour_csr()
    for _ in range(10):
        s.integrator.integrate(1e-4)
    assert s.integrator.step_stats()["graph_steps"] >= 1
    host = {k: pa.get(k) for k in ("x", "y", "z", "h")}
    off, idx = oracle.neighbors(host, host, particles.cell_manager.cell_size, same=True)
    goff, gidx = loc.neighbour_csr()
    assert np.array_equal(goff, off) and np.array_equal(gidx, idx)


def test_hooks_attached_after_recording_run_every_step(monkeypatch):
    """A rates hook (the learned closure's interface) attached after the
    step was recorded is called at every later step: the recorded step is
    not replayed while hooks are attached, and is recorded afresh once they
    are gone."""
    _need_gpu()
    monkeypatch.setenv("PYSPH_GB300_GRAPHS", "1")
    props = W.cube_lattice(8000, seed=36)
    s, particles = W.setup_cube(API, props)
    integ = s.integrator
    for _ in range(4):
        integ.integrate(1e-4)
    assert integ.step_stats() is not None

    class Counter:
        calls = 0

        def before_rates(self, integ, stage, terms):
            Counter.calls += 1
            return terms

        def after_rates(self, integ, stage, acc):
            pass

    stage = next(st for st in integ.stages if getattr(st, "hooks", None) is not None)
    hook = Counter()
    stage.hooks.append(hook)
    for _ in range(3):
        before = Counter.calls
        integ.integrate(1e-4)
        assert Counter.calls > before
    assert integ.step_stats() is None
    stage.hooks.remove(hook)
    done = Counter.calls
    for _ in range(3):
        integ.integrate(1e-4)
    assert Counter.calls == done
    assert integ.step_stats() is not None
