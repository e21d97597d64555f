"""Host-side behaviour of the drop-in API that needs no GPU: operation
expansion, calc validation errors, the integrator's stage plan."""
import numpy as np
import pytest
import torch

import pysph_gb300
from pysph_gb300 import workloads as W

API = pysph_gb300.api()
base, sph, solver = API.base, API.sph, API.solver


def _pa(n=10, name="fluid", type=0):
    x = np.linspace(0, 1, n)
    return base.get_particle_array(name=name, type=type, x=x, h=np.full(n, 0.2))


def test_get_particle_array_defaults():
    pa = _pa()
    for p in ("x", "y", "z", "u", "v", "w", "m", "h", "p", "e", "rho", "cs", "idx", "tag"):
        assert pa.has_array(p)
    assert pa.get_number_of_particles() == 10
    assert np.all(pa.get("m") == 1.0) and np.all(pa.get("rho") == 1.0)
    np.testing.assert_array_equal(pa.get("idx"), np.arange(10))
    assert pa.num_real_particles == 10
    with pytest.raises(AttributeError):
        pa.get("nope")


def test_set_marks_dirty_only_for_positions():
    pa = _pa()
    pa.set_dirty(False)
    pa.set(u=np.ones(10))
    assert not pa.is_dirty
    pa.set(x=np.zeros(10))
    assert pa.is_dirty


def test_remove_particles_swaps_with_last():
    pa = _pa(6)
    pa.remove_particles(base.LongArray(0) if False else np.array([1]))
    np.testing.assert_array_equal(pa.get("idx"), [0, 5, 2, 3, 4])


def test_calc_checks_raise_value_error():
    a = _pa()
    b = _pa(name="other")
    particles = base.Particles(arrays=[a, b])
    k = base.CubicSplineKernel(dim=1)
    f = sph.SPHRho.get_func(a, a)
    with pytest.raises(ValueError, match="One sph function is needed per source"):
        sph.SPHCalc(particles, [a, b], a, k, [f], ["rho"])
    with pytest.raises(ValueError, match="Number of updates"):
        sph.SPHCalc(particles, [a], a, k, [f], ["rho", "p"])
    with pytest.raises(ValueError, match="same type"):
        sph.SPHCalc(particles, [a, b], a, k,
                    [f, sph.SPHPressureGradient.get_func(b, a)], ["rho"])
    with pytest.raises(ValueError, match="SPHFunction.source"):
        sph.SPHCalc(particles, [b], a, k, [f], ["rho"])


def test_avisc_never_stores_eta():
    a = _pa()
    f = sph.MonaghanArtificialVsicosity.withargs(alpha=0.3, beta=0.2, eta=0.7).get_func(a, a)
    assert f.eta == 0.0 and f.alpha == 0.3 and f.num_outputs == 3


def test_unsupported_functions_raise():
    a = _pa()
    with pytest.raises(NotImplementedError):
        sph.XSPHDensityRate.withargs().get_func(a, a)
    with pytest.raises(NotImplementedError):
        base.QuinticSplineKernel(dim=2)


def test_operation_expansion_and_stage_plan():
    fl, wl = W.dam_break(dx=0.1)
    s, particles = W.setup_dam_break(API, fl, wl, dx=0.1, c0=W.dam_break_c0())
    integ = s.integrator
    ids = [c.id for c in integ.calcs]
    assert ids == ["eos_fluid", "density_fluid", "pgrad_fluid", "avisc_fluid",
                   "bforce_fluid", "gravity_fluid", "step_fluid"]
    kinds = [type(st).__name__ for st in integ.stages]
    # Tait precedes SPHRho, so it is not fused; the integrating run is one stage
    assert kinds == ["TaitStage", "DensityStage", "RatesStage"]
    rs = integ.stages[-1]
    assert rs.gravity == (0.0, -9.81, 0.0) and rs.add_velocity
    by_src = {t["src"].name: t["kinds"] for t in rs.terms}
    assert by_src == {"fluid": {"pgrad", "avisc"}, "boundary": {"bforce"}}
    assert integ.k_props["pgrad_fluid"]["k2"] == ["_k2_u20", "_k2_v21"]
    fluid = particles.arrays[0]
    for p in ("_u_0", "_v_0", "_x_0", "_rate1_u", "_rate2_y"):
        assert fluid.has_array(p)


def test_drop_plan_fuses_density_and_tait():
    s, _ = W.setup_drop(API, W.elliptical_drop(dx=0.1))
    st = s.integrator.stages
    assert [type(x).__name__ for x in st] == ["DensityStage", "RatesStage"]
    assert st[0].tait is not None
    assert st[1].terms[0]["kinds"] == {"pgrad", "avisc", "xsph"}


def test_compute_without_gpu_raises():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    s, _ = W.setup_drop(API, W.elliptical_drop(dx=0.1))
    with pytest.raises(RuntimeError, match="CUDA device"):
        s.integrator.integrate(1e-5)


def test_fluid_solver_plan_integrates_rho():
    s, particles = W.setup_fluid_solver(API, W.circular_patch(dx=0.2))
    st = s.integrator.stages
    assert [type(x).__name__ for x in st] == ["TaitStage", "RatesStage"]
    rates = st[1]
    assert set(rates.props) == {"rho", "u", "v", "w", "x", "y"}
    assert len(rates.terms) == 1
    assert rates.terms[0]["kinds"] == {"drho", "momentum", "xsph"}
    assert rates.terms[0]["eta"] == 0.1


def test_multistage_integrators_rate_arrays():
    for scheme, nsteps in (("rk4", 4), ("pc", 2), ("leapfrog", 2)):
        s, particles = W.setup_cube(API, W.cube_lattice(512), integrator=scheme)
        integ = s.integrator
        assert integ.nsteps == nsteps
        fluid = particles.arrays[0]
        for l in range(1, nsteps + 1):
            for p in ("u", "v", "w", "x", "y", "z"):
                assert fluid.has_array("_rate%d_%s" % (l, p)), (scheme, l, p)
        assert not fluid.has_array("_rate%d_u" % (nsteps + 1))


def test_leapfrog_plans_velocity_and_position_calcs_apart():
    """integrator.py:893-912 evaluates non-position and position calcs in
    separate passes, so they never share a rates launch."""
    s, _ = W.setup_cube(API, W.cube_lattice(512), integrator="leapfrog")
    integ = s.integrator
    assert [type(x).__name__ for x in integ.stages] == ["DensityStage", "RatesStage", "RatesStage"]
    vel, pos = integ.stages[1], integ.stages[2]
    assert set(vel.props) == {"u", "v", "w"} and not vel.add_velocity
    assert set(pos.props) == {"x", "y", "z"} and pos.add_velocity and not pos.terms
    assert integ._stages_for(integ.ncalcs) == integ.stages[:2]
    assert integ._stages_for(integ.pcalcs) == integ.stages[2:]
    # the RK2 plan of the same calcs fuses them into one rates launch
    s2, _ = W.setup_cube(API, W.cube_lattice(512), integrator="rk2")
    assert [type(x).__name__ for x in s2.integrator.stages] == ["DensityStage", "RatesStage"]


def test_leapfrog_2d_index_error_before_any_work():
    s, _ = W.setup_drop(API, W.elliptical_drop(dx=0.1), integrator="leapfrog")
    with pytest.raises(IndexError):
        s.integrator.integrate(1e-5)


def test_variable_h_switches_the_cell_manager_to_the_symmetric_relation():
    props = W.jitter_h(W.elliptical_drop(dx=0.1))
    pa = base.get_particle_array(name="fluid", **props)
    particles = base.Particles(arrays=[pa], variable_h=True, update_particles=False)
    assert particles.cell_manager.symmetric
    pb = base.get_particle_array(name="fluid", **props)
    assert not base.Particles(arrays=[pb], update_particles=False).cell_manager.symmetric


def test_periodic_domain_translate_rules():
    """base/cell.pyx:1568-1598: an axis spanning exactly 2000 is not periodic."""
    d = base.PeriodicDomain(xmin=-0.2, xmax=1.0)
    assert d.xtranslate == pytest.approx(1.2) and d.ytranslate == 0.0 and d.ztranslate == 0.0
    pa = base.get_particle_array(name="f", x=np.linspace(0, 1, 5), h=np.full(5, 0.1))
    with pytest.raises(NotImplementedError):
        base.CellManager(arrays_to_bin=[pa], periodic_domain=base.PeriodicDomain(ymin=0, ymax=1),
                         initialize=False)


def test_staged_transfers_check_their_arguments():
    pa = base.get_particle_array(name="f", x=np.zeros(4), y=np.zeros(4))
    with pytest.raises(ValueError):
        pa.upload()
    with pytest.raises(ValueError):
        pa.download()
    with pytest.raises(AttributeError):
        pa.upload(q=np.zeros(4))
    if not torch.cuda.is_available():
        # host-resident arrays (no GPU): the staged forms need device arrays
        with pytest.raises(RuntimeError):
            pa.upload(x=np.ones(4))
        with pytest.raises(RuntimeError):
            pa.download("x")


def test_base5_cell_offset_decode_is_exact():
    """The base-5 list-entry code (stencil half-width 2 above 2^23 source
    particles): (dx+2) + 5 (dy+2) + 25 (dz+2), decoded with c / 25 =
    (c 1311) >> 15 and r / 5 = (r 13) >> 6 -- exact for every code."""
    seen = set()
    for dz in range(-2, 3):
        for dy in range(-2, 3):
            for dx in range(-2, 3):
                row = 2 + 5 * (dy + 2) + 25 * (dz + 2)     # Code<4>::row
                c = row + dx
                assert 0 <= c < 128
                z = (c * 1311) >> 15
                r = c - 25 * z
                y = (r * 13) >> 6
                x = r - 5 * y
                assert (x - 2, y - 2, z - 2) == (dx, dy, dz)
                seen.add(c)
    assert len(seen) == 125


def test_list_skin_defaults(monkeypatch):
    """The list skin a neighbour structure starts with and the integrators'
    rule for growing it: doubling below 500 000 particles, none from there up
    or when the environment fixes the skin."""
    from pysph_gb300 import tuning
    monkeypatch.delenv("PYSPH_GB300_SKIN", raising=False)
    assert tuning.list_skin() == tuning.DEFAULT_SKIN
    assert tuning.skin_growth(tuning.GRAPH_MAX_PARTICLES - 1) == (
        tuning.SKIN_WINDOW, tuning.SKIN_WINDOW // 4, 2.0, tuning.SKIN_MAX)
    assert tuning.skin_growth(tuning.GRAPH_MAX_PARTICLES) is None
    monkeypatch.setenv("PYSPH_GB300_SKIN", "0.05")
    assert tuning.list_skin() == 0.05
    assert tuning.skin_growth(10) is None


def test_guard_stats_report_the_spread_of_window_errors():
    """GuardedRunner.stats(): windows, checks, kept and fallbacks, and the
    smallest, median and largest normwise error of the checked windows."""
    from pysph_gb300 import learned as L
    r = object.__new__(L.GuardedRunner)
    r.windows, r.checks, r.kept, r.fallbacks = 7, 5, 2, 3
    r.errors = [3e-3, 2e-4, 5e-4, 9e-4, 4e-2]
    r.max_err, r.max_err_maxrel = max(r.errors), 0.1
    st = r.stats()
    assert (st["windows"], st["checks"], st["kept"], st["fallbacks"]) == (7, 5, 2, 3)
    assert st["fallback_rate"] == 0.6
    assert st["min_normwise_density_error"] == 2e-4
    assert st["median_normwise_density_error"] == 9e-4
    assert st["max_normwise_density_error"] == 4e-2
    r.errors, r.checks = [], 0
    st = r.stats()
    assert st["fallback_rate"] is None and st["median_normwise_density_error"] is None
