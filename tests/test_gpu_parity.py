"""GPU parity: the CUDA path against the reference's golden fixtures and the
oracle.

Tolerance: neighbour sets bit-exact (as index sets, self last); every
floating-point field within ``TOL = 1e-5`` normwise relative error
(``max|gpu - ref| / max|ref|``), the FP32 pair-sum contract.  State after a
step is compared through its increment (``x_out - x_in``), which is what the
FP32 rates determine.
"""
import numpy as np
import pytest
import torch

import oracle
import pysph_gb300
from golden_util import csr_sets, inputs, load, normwise
from pysph_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-5
API = pysph_gb300.api()
base, sph, solver = API.base, API.sph, API.solver


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")


def _particles(g, specs):
    arrays = []
    for name, ptype in specs:
        arrays.append(base.get_particle_array(name=name, type=ptype, **inputs(g, name)))
    return arrays, base.Particles(arrays=arrays)


def _locator_sets(particles, src, dst):
    loc = particles.nnps_manager.get_neighbor_particle_locator(src, dst, 2.0)
    off, idx = loc.neighbour_csr()
    return off, idx


@pytest.mark.parametrize("name", ["drop_step", "cube_step"])
def test_neighbour_sets_bit_exact(name):
    _need_gpu()
    g = load(name)
    (pa,), particles = _particles(g, [("fluid", base.ParticleType.Fluid)])
    off, idx = _locator_sets(particles, pa, pa)
    ro, ri = g["nbr_fluid_fluid_offsets"], g["nbr_fluid_fluid_index"]
    assert csr_sets(off, idx) == csr_sets(ro, ri)
    np.testing.assert_array_equal(idx[off[1:] - 1], np.arange(len(off) - 1))
    # the locator API returns the same lists
    loc = particles.nnps_manager.get_neighbor_particle_locator(pa, pa, 2.0)
    for i in (0, 7, len(off) // 2, len(off) - 2):
        lst = loc.py_get_nearest_particles(i).get_npy_array()
        assert set(lst.tolist()) == set(ri[ro[i]:ro[i + 1]].tolist())
        assert lst[-1] == i


def test_dam_neighbour_sets_bit_exact():
    _need_gpu()
    g = load("dam_step")
    (fl, wl), particles = _particles(g, [("fluid", base.ParticleType.Fluid),
                                         ("boundary", base.ParticleType.Solid)])
    for src, key in ((fl, "fluid"), (wl, "boundary")):
        off, idx = _locator_sets(particles, src, fl)
        assert csr_sets(off, idx) == csr_sets(g["nbr_fluid_%s_offsets" % key],
                                              g["nbr_fluid_%s_index" % key])


def test_square4_functions():
    _need_gpu()
    g = load("square4")
    props = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    pa = base.get_particle_array(name="test", tmpx=np.zeros(4), tmpy=np.zeros(4),
                                 tmpz=np.zeros(4), **props)
    particles = base.Particles(arrays=[pa])
    kern = base.CubicSplineKernel(dim=2)
    for name, fn, ups in (
            ("rho", sph.SPHRho.withargs(), ["tmpx"]),
            ("pgrad", sph.SPHPressureGradient.withargs(dim=2), ["tmpx", "tmpy"]),
            ("avisc", sph.MonaghanArtificialVsicosity.withargs(alpha=1.0, beta=1.0),
             ["tmpx", "tmpy", "tmpz"]),
            ("xsph", sph.XSPHCorrection.withargs(eps=0.5, dim=2), ["tmpx", "tmpy"])):
        calc = sph.SPHCalc(particles, [pa], pa, kern, [fn.get_func(pa, pa)], ups)
        calc.sph(*ups)
        for k, upn in enumerate(ups):
            ref = g["%s_%d" % (name, k)]
            got = pa.get(upn)
            assert np.abs(got - ref).max() <= TOL * max(np.abs(ref).max(), 1.0), (name, k)


def test_drop_per_function_parity():
    """Each SPH function of the drop on the reference's own input state."""
    _need_gpu()
    g = load("drop_step")
    inp = inputs(g, "fluid")
    n = len(inp["x"])
    pa = base.get_particle_array(name="fluid", type=base.ParticleType.Fluid,
                                 t0=np.zeros(n), t1=np.zeros(n), t2=np.zeros(n), **inp)
    particles = base.Particles(arrays=[pa])
    k2 = base.CubicSplineKernel(dim=2)

    def calc(fn, ups, srcs=(pa,)):
        funcs = [fn.get_func(s, pa) for s in srcs]
        return sph.SPHCalc(particles, list(srcs), pa, k2, funcs, ups)

    calc(sph.SPHRho.withargs(), ["rho"]).sph("rho")
    assert normwise(pa.get("rho"), g["eval1_fluid_rho"]) < TOL
    c = sph.SPHCalc(particles, [], pa, k2, [sph.TaitEquation.withargs(co=1400.0, ro=1.0).get_func(pa, pa)],
                    ["p", "cs"])
    c.sph("p", "cs")
    assert normwise(pa.get("p"), g["eval1_fluid_p"]) < TOL
    assert normwise(pa.get("cs"), g["eval1_fluid_cs"]) < TOL
    calc(sph.SPHPressureGradient.withargs(dim=2), ["u", "v"]).sph("t0", "t1")
    assert normwise(pa.get("t0"), g["eval1_k_pgrad_fluid_u"]) < TOL
    assert normwise(pa.get("t1"), g["eval1_k_pgrad_fluid_v"]) < TOL
    calc(sph.MonaghanArtificialVsicosity.withargs(alpha=0.01, beta=0.0),
         ["u", "v", "w"]).sph("t0", "t1", "t2")
    assert normwise(pa.get("t0"), g["eval1_k_avisc_fluid_u"]) < TOL
    assert normwise(pa.get("t1"), g["eval1_k_avisc_fluid_v"]) < TOL
    calc(sph.XSPHCorrection.withargs(eps=0.5, dim=2), ["x", "y"]).sph("t0", "t1")
    assert normwise(pa.get("t0"), g["eval1_k_xsph_fluid_x"]) < TOL
    assert normwise(pa.get("t1"), g["eval1_k_xsph_fluid_y"]) < TOL


def _check_step(g, arrays, evals, k_groups):
    """Compare rates of every eval and the state increment with the reference."""
    for pa in arrays:
        nm = pa.name
        for p in ("rho", "p", "cs"):
            key = "out_%s_%s" % (nm, p)
            if key in g and np.abs(g[key]).max() > 0:
                assert normwise(pa.get(p), g[key]) < TOL, key
        for p in ("x", "y", "z", "u", "v", "w"):
            key = "out_%s_%s" % (nm, p)
            if key not in g:
                continue
            d_ref = g[key] - g["in_%s_%s" % (nm, p)]
            if np.abs(d_ref).max() == 0:
                continue
            d_got = pa.get(p) - g["in_%s_%s" % (nm, p)]
            assert normwise(d_got, d_ref) < TOL, (key, normwise(d_got, d_ref))
    # summed rates of each evaluation
    pa = arrays[0]
    for e in range(1, evals + 1):
        for prop, calcs in k_groups.items():
            ref = sum(g["eval%d_k_%s_fluid_%s" % (e, c, prop)] for c in calcs)
            got = pa.get("_rate%d_%s" % (e, prop))
            assert normwise(got, ref) < TOL, (e, prop, normwise(got, ref))


def test_drop_euler_step():
    _need_gpu()
    g = load("drop_step")
    s, particles = W.setup_drop(API, inputs(g, "fluid"))
    s.integrator.integrate(float(g["dt"]))
    _check_step(g, particles.arrays, 1, {"u": ["pgrad", "avisc"], "v": ["pgrad", "avisc"],
                                         "x": ["step", "xsph"], "y": ["step", "xsph"]})


def test_drop_ten_steps_trajectory():
    _need_gpu()
    g = load("drop_traj10")
    inp = inputs(g, "fluid")
    s, particles = W.setup_drop(API, inp)
    for _ in range(int(g["steps"])):
        s.integrator.integrate(float(g["dt"]))
    pa = particles.arrays[0]
    for p in ("x", "y", "u", "v"):
        d_ref = g["final_" + p] - inp[p]
        assert normwise(pa.get(p) - inp[p], d_ref) < 1e-4, p
    for p in ("rho", "p"):
        assert normwise(pa.get(p), g["final_" + p]) < 1e-4, p


def test_dam_rk2_step():
    _need_gpu()
    g = load("dam_step")
    fl, wl = inputs(g, "fluid"), inputs(g, "boundary")
    s, particles = W.setup_dam_break(API, fl, wl, dx=float(g["dx"]), c0=float(g["c0"]))
    s.integrator.integrate(float(g["dt"]))
    _check_step(g, particles.arrays[:1], 2,
                {"u": ["pgrad", "avisc", "bforce", "gravity"],
                 "v": ["pgrad", "avisc", "bforce", "gravity"], "x": ["step"], "y": ["step"]})


def test_cube_rk2_step():
    _need_gpu()
    g = load("cube_step")
    s, particles = W.setup_cube(API, inputs(g, "fluid"))
    s.integrator.integrate(float(g["dt"]))
    _check_step(g, particles.arrays, 2,
                {"u": ["pgrad", "avisc"], "v": ["pgrad", "avisc"], "w": ["pgrad", "avisc"],
                 "x": ["step"], "y": ["step"], "z": ["step"]})


@pytest.mark.parametrize("n,subdiv", [(32768, 1), (32768, 2), (64000, 3)])
def test_cube_vs_oracle(n, subdiv, monkeypatch):
    """Larger 3D lattices against the C oracle, for every cell subdivision."""
    _need_gpu()
    monkeypatch.setenv("PYSPH_GB300_SUBDIV", str(subdiv))
    props = W.cube_lattice(n, seed=3)
    s, particles = W.setup_cube(API, props)
    dt = 1e-4
    s.integrator.integrate(dt)
    pa = particles.arrays[0]
    prob = oracle.Problem({"fluid": props}, oracle.cube_ops(), dim=3)
    prob.integrate_rk2(dt)
    ref = prob.arrays["fluid"]
    for p in ("rho", "p", "cs"):
        assert normwise(pa.get(p), ref[p]) < TOL, p
    for p in ("x", "y", "z", "u", "v", "w"):
        assert normwise(pa.get(p) - props[p], ref[p] - props[p]) < TOL, p


def test_jump_tolerance_raises():
    """A particle moving more than one cell between builds raises
    RuntimeError, as CellManager.check_jump_tolerance does."""
    _need_gpu()
    props = W.elliptical_drop(dx=0.1)
    pa = base.get_particle_array(name="fluid", **props)
    particles = base.Particles(arrays=[pa])
    cs = particles.cell_manager.cell_size
    x = pa.get("x")
    x[3] += 2.5 * cs
    pa.set(x=x)
    with pytest.raises(RuntimeError, match="more than one cell"):
        particles.update()


def test_non_real_tags_get_zero():
    _need_gpu()
    props = W.elliptical_drop(dx=0.05)
    n = len(props["x"])
    tag = np.zeros(n, np.int64)
    tag[::7] = 1   # Dummy particles: still neighbours, never destinations
    pa = base.get_particle_array(name="fluid", **props)
    pa.add_property({"name": "tag", "data": tag, "type": "long"})
    pa.align_particles()
    particles = base.Particles(arrays=[pa])
    k2 = base.CubicSplineKernel(dim=2)
    sph.SPHCalc(particles, [pa], pa, k2, [sph.SPHRho.get_func(pa, pa)], ["rho"]).sph("rho")
    rho = pa.get("rho", only_real_particles=False)
    t = pa.get("tag", only_real_particles=False)
    assert np.all(rho[t != 0] == 0)
    host = {k: pa.get(k, only_real_particles=False) for k in ("x", "y", "z", "h", "m")}
    host["tag"] = t
    off, idx = oracle.neighbors(host, host, particles.cell_manager.cell_size, same=True)
    ref = oracle.pair_sum("rho", host, host, off, idx, 2)[0]
    assert normwise(rho, ref) < TOL


def test_invariants_mass_exact():
    _need_gpu()
    props = W.cube_lattice(8000)
    s, particles = W.setup_cube(API, props)
    inv0 = particles.invariants()
    for _ in range(3):
        s.integrator.integrate(1e-4)
    inv1 = particles.invariants()
    assert inv1["mass"] == inv0["mass"]
    assert inv1["count"] == len(props["x"])
    assert abs(inv0["mass"] - props["m"].sum()) <= 1e-12 * props["m"].sum()


def test_list_overflow_retraversal_matches():
    """Destinations with more neighbours than the list capacity are
    completed by re-traversal; results must not change."""
    _need_gpu()
    import subprocess
    import sys
    code = r'''
import sys, numpy as np
sys.path.insert(0, ".")
import oracle, pysph_gb300
from pysph_gb300 import workloads as W
from tests.golden_util import normwise
props = W.cube_lattice(8000, seed=5)
s, particles = W.setup_cube(pysph_gb300.api(), props)
s.integrator.integrate(1e-4)
pa = particles.arrays[0]
prob = oracle.Problem({"fluid": props}, oracle.cube_ops(), dim=3)
prob.integrate_rk2(1e-4)
for p in ("rho", "p"):
    assert normwise(pa.get(p), prob.arrays["fluid"][p]) < 1e-5, p
for p in ("x", "u", "w"):
    assert normwise(pa.get(p) - props[p], prob.arrays["fluid"][p] - props[p]) < 1e-5, p
print("ok")
'''
    import os
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    # both kernel families: the list-streaming passes and the brick-staged ones
    for bricks in ("0", "1"):
        env = dict(os.environ, SPH_LIST_CAP="7", PYSPH_GB300_BRICKS=bricks)
        r = subprocess.run([sys.executable, "-c", code], cwd=root, env=env, capture_output=True,
                           text=True, timeout=600)
        assert r.returncode == 0 and "ok" in r.stdout, (bricks, r.stderr[-3000:])


def test_square4_momentum_and_density_rate():
    _need_gpu()
    g = load("square4_momentum")
    props = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    pa = base.get_particle_array(name="test", tmpx=np.zeros(4), tmpy=np.zeros(4),
                                 tmpz=np.zeros(4), **props)
    particles = base.Particles(arrays=[pa])
    kern = base.CubicSplineKernel(dim=2)
    for name, fn, ups in (
            ("momentum", sph.MomentumEquation.withargs(alpha=1.0, beta=1.0, eta=0.1),
             ["tmpx", "tmpy", "tmpz"]),
            ("drho", sph.SPHDensityRate.withargs(), ["tmpx"])):
        calc = sph.SPHCalc(particles, [pa], pa, kern, [fn.get_func(pa, pa)], ups)
        calc.sph(*ups)
        for k, upn in enumerate(ups):
            ref = g["%s_%d" % (name, k)]
            got = pa.get(upn)
            assert np.abs(got - ref).max() <= TOL * max(np.abs(ref).max(), 1.0), (name, k)


def test_fluid_solver_rk2_step():
    """The reference FluidSolver recipe: continuity density rate,
    MomentumEquation, stepping and XSPH in one rates launch per evaluation."""
    _need_gpu()
    g = load("fluid_step")
    p_in = inputs(g, "fluid")
    s, particles = W.setup_fluid_solver(API, p_in)
    s.integrator.integrate(float(g["dt"]))
    pa = particles.arrays[0]
    _check_step(g, [pa], 2, {"rho": ["density"], "u": ["mom"], "v": ["mom"],
                             "x": ["step", "xsph"], "y": ["step", "xsph"]})
    d_ref = g["out_fluid_rho"] - p_in["rho"]
    assert normwise(pa.get("rho") - p_in["rho"], d_ref) < TOL


# -- RK4, predictor-corrector and leap-frog (solver/integrator.py:650-912) ---

DROP_K = {"u": ["pgrad", "avisc"], "v": ["pgrad", "avisc"], "x": ["step", "xsph"],
          "y": ["step", "xsph"]}
FLUID_K = {"rho": ["density"], "u": ["mom"], "v": ["mom"], "x": ["step", "xsph"],
           "y": ["step", "xsph"]}


def _check_final(g, pa, inp):
    """State after the fixture's ``steps`` steps (increments for x, v)."""
    for p in ("x", "y", "u", "v"):
        d_ref = g["final_" + p] - inp[p]
        assert normwise(pa.get(p) - inp[p], d_ref) < 1e-4, p
    for p in ("rho", "p"):
        assert normwise(pa.get(p), g["final_" + p]) < 1e-4, p


@pytest.mark.parametrize("scheme", ["rk4", "pc"])
def test_drop_multistage_steps(scheme):
    _need_gpu()
    g = load("drop_" + scheme)
    inp = inputs(g, "fluid")
    s, particles = W.setup_drop(API, inp, integrator=scheme)
    dt = float(g["dt"])
    s.integrator.integrate(dt)
    _check_step(g, particles.arrays, int(g["n_evals"]), DROP_K)
    for _ in range(int(g["steps"]) - 1):
        s.integrator.integrate(dt)
    _check_final(g, particles.arrays[0], inp)


@pytest.mark.parametrize("scheme", ["rk4", "pc"])
def test_fluid_solver_multistage_steps(scheme):
    _need_gpu()
    g = load("fluid_" + scheme)
    inp = inputs(g, "fluid")
    s, particles = W.setup_fluid_solver(API, inp, integrator=scheme)
    dt = float(g["dt"])
    s.integrator.integrate(dt)
    pa = particles.arrays[0]
    _check_step(g, [pa], int(g["n_evals"]), FLUID_K)
    d_ref = g["out_fluid_rho"] - inp["rho"]
    assert normwise(pa.get("rho") - inp["rho"], d_ref) < TOL
    for _ in range(int(g["steps"]) - 1):
        s.integrator.integrate(dt)
    _check_final(g, pa, inp)


def test_cube_leapfrog_step():
    """Velocity calcs at the start, the position calc once on the predicted
    velocities (plus the h^2/2 F0 correction), velocity calcs again after
    the neighbour update."""
    _need_gpu()
    g = load("cube_leapfrog")
    s, particles = W.setup_cube(API, inputs(g, "fluid"), integrator="leapfrog")
    s.integrator.integrate(float(g["dt"]))
    pa = particles.arrays[0]
    _check_step(g, [pa], 0, {})
    for prop in "uvw":
        for e, lvl in ((1, 1), (3, 2)):
            ref = sum(g["eval%d_k_%s_fluid_%s" % (e, c, prop)] for c in ("pgrad", "avisc"))
            assert normwise(pa.get("_rate%d_%s" % (lvl, prop)), ref) < TOL, (e, prop)
    for prop in "xyz":
        assert normwise(pa.get("_rate1_" + prop), g["eval2_k_step_fluid_" + prop]) < TOL


def test_leapfrog_2d_drop_raises_index_error():
    """The reference's add_correction_for_position indexes the position
    calc's two updates with the three outputs of the 2D Monaghan viscosity
    and raises IndexError; so does the GPU integrator, before any work."""
    _need_gpu()
    g = load("drop_step")
    s, particles = W.setup_drop(API, inputs(g, "fluid"), integrator="leapfrog")
    x0 = particles.arrays[0].get("x").copy()
    with pytest.raises(IndexError):
        s.integrator.integrate(1e-5)
    np.testing.assert_array_equal(particles.arrays[0].get("x"), x0)


# -- variable h: Particles(variable_h=True), VarHNbrParticleLocator ------------

def test_variable_h_neighbour_sets_bit_exact():
    """The symmetric union (base/nnps.pyx:654-749) as index sets, from the
    exported lists of the device build."""
    _need_gpu()
    g = load("drop_varh")
    pa = base.get_particle_array(name="fluid", type=base.ParticleType.Fluid,
                                 **inputs(g, "fluid"))
    particles = base.Particles(arrays=[pa], variable_h=True)
    off, idx = _locator_sets(particles, pa, pa)
    ro, ri = g["nbr_fluid_fluid_offsets"], g["nbr_fluid_fluid_index"]
    assert csr_sets(off, idx) == csr_sets(ro, ri)
    loc = particles.nnps_manager.get_neighbor_particle_locator(pa, pa, 2.0)
    assert type(loc).__name__ == "VarHNbrParticleLocator"
    # fixed-h lists of the same particles are a strict subset
    pb = base.get_particle_array(name="fluid", type=base.ParticleType.Fluid,
                                 **inputs(g, "fluid"))
    o2, i2 = _locator_sets(base.Particles(arrays=[pb]), pb, pb)
    assert o2[-1] < off[-1]


@pytest.mark.parametrize("skin", ["0", "0.03"])
def test_variable_h_euler_step(skin, monkeypatch):
    """One Euler step of the drop with per-particle h over the symmetric
    neighbour relation (pair sums at the mean h of each pair)."""
    _need_gpu()
    monkeypatch.setenv("PYSPH_GB300_SKIN", skin)
    g = load("drop_varh")
    s, particles = W.setup_drop(API, inputs(g, "fluid"), variable_h=True)
    s.integrator.integrate(float(g["dt"]))
    _check_step(g, particles.arrays, 1, DROP_K)


# -- periodic x (PeriodicDomain, base/cell.pyx:1277-1376) ---------------------

def _periodic_particles(g):
    n = int(g["n_real"])
    props = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    pa = base.get_particle_array(name="fluid", type=base.ParticleType.Fluid,
                                 tmpx=np.zeros(n), tmpy=np.zeros(n), tmpz=np.zeros(n), **props)
    dom = base.PeriodicDomain(xmin=float(g["xmin"]), xmax=float(g["xmax"]))
    return pa, base.Particles(arrays=[pa], periodic_domain=dom)


def test_periodic_neighbour_sets_bit_exact():
    """The reference's lists over real and ghost particles, ghosts mapped to
    the particle they copy, against the device build's images."""
    _need_gpu()
    g = load("periodic")
    n = int(g["n_real"])
    pa, particles = _periodic_particles(g)
    assert pa.get_number_of_particles() == n     # no ghost particles appended
    origin = g["ghost_origin"]
    ref = [{(j if j < n else int(origin[j - n])) for j in s}
           for s in csr_sets(g["nbr_offsets"], g["nbr_index"])]
    off, idx = _locator_sets(particles, pa, pa)
    assert csr_sets(off, idx) == ref


def test_periodic_pair_functions():
    """Every pair function on the initial state (the reference's ghosts
    still carry their originals' state there)."""
    _need_gpu()
    g = load("periodic")
    pa, particles = _periodic_particles(g)
    kern = base.CubicSplineKernel(dim=2)
    for name, fn, ups in (
            ("pgrad", sph.SPHPressureGradient.withargs(dim=2), ["tmpx", "tmpy"]),
            ("avisc", sph.MonaghanArtificialVsicosity.withargs(alpha=1.0, beta=1.0),
             ["tmpx", "tmpy", "tmpz"]),
            ("xsph", sph.XSPHCorrection.withargs(eps=0.5, dim=2), ["tmpx", "tmpy"]),
            ("rho", sph.SPHRho.withargs(), ["tmpx"])):
        calc = sph.SPHCalc(particles, [pa], pa, kern, [fn.get_func(pa, pa)], ups)
        calc.sph(*ups)
        for k, upn in enumerate(ups):
            ref = g["%s_%d" % (name, k)]
            assert normwise(pa.get(upn), ref) < TOL, (name, k, normwise(pa.get(upn), ref))


def test_periodic_step_after_crossing_vs_oracle():
    """Ten Euler steps of the drop operations on a jittered strip with a
    uniform drift that carries the last column across the periodic end; then one
    more step from that shared state, GPU against the oracle's periodic
    images (per-step parity, 1e-5).  The reference itself cannot run this:
    its ghosts are re-appended at every update and zeroed by every calc."""
    _need_gpu()
    # jittered lattice: on the exact lattice the pressure forces cancel to
    # ~1e-4 of their terms and FP32 sums cannot carry the x rate to 1e-5
    props = W.periodic_strip(vel_std=0.1, jitter=0.1)
    props["u"] = props["u"] + 50.0
    dom = (0.0, 1.0)
    s, particles = W.setup_drop(API, props, c0=10.0,
                                periodic_domain=base.PeriodicDomain(xmin=dom[0], xmax=dom[1]))
    dt = 1e-4
    for _ in range(10):
        s.integrator.integrate(dt)
    pa = particles.arrays[0]
    assert pa.get("x").max() > dom[1]             # some particles left the period
    state = {k: pa.get(k).copy() for k in props}
    prob = oracle.Problem({"fluid": state}, oracle.drop_ops(c0=10.0), 2, periodic=dom)
    prob.integrate_euler(dt)
    s.integrator.integrate(dt)
    for p in ("x", "y", "u", "v"):
        d_ref = prob.arrays["fluid"][p] - state[p]
        assert normwise(pa.get(p) - state[p], d_ref) < TOL, (p, normwise(pa.get(p) - state[p], d_ref))
    for p in ("rho", "p"):
        assert normwise(pa.get(p), prob.arrays["fluid"][p]) < TOL, p


def test_periodic_trajectory_vs_oracle():
    """A gentle strip (c0 = 1, small velocities, drift across the end):
    ten Euler steps against the oracle within 1e-4."""
    _need_gpu()
    props = W.periodic_strip(vel_std=0.1, c0=1.0, jitter=0.1)
    props["u"] = props["u"] + 50.0
    dom = (0.0, 1.0)
    s, particles = W.setup_drop(API, props, c0=1.0,
                                periodic_domain=base.PeriodicDomain(xmin=dom[0], xmax=dom[1]))
    prob = oracle.Problem({"fluid": props}, oracle.drop_ops(c0=1.0), 2, periodic=dom)
    for _ in range(10):
        s.integrator.integrate(1e-4)
        prob.integrate_euler(1e-4)
    pa = particles.arrays[0]
    for p in ("x", "y", "u", "v"):
        d_ref = prob.arrays["fluid"][p] - props[p]
        assert normwise(pa.get(p) - props[p], d_ref) < 1e-4, (p, normwise(pa.get(p) - props[p], d_ref))


# -- Solver.solve output (solver.py:457-538) ------------------------------------

def test_solver_output_files_match_reference(tmp_path):
    """The .npz files Solver.solve writes: the same names, keys and values
    as the reference's (dt, cell_size, np and the print properties)."""
    _need_gpu()
    g = load("drop_output")
    props = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    s, particles = W.setup_drop(API, props)
    s.set_time_step(1e-5)
    s.set_final_time(3 * 1e-5 * (1 - 1e-9))
    s.set_print_freq(1)
    s.set_output_printing_level(False)
    s.set_output_directory(str(tmp_path))
    s.set_output_fname("drop")
    s.solve()
    names = sorted(p.name for p in tmp_path.iterdir())
    assert names == list(g["files"])
    for k, f in enumerate(names):
        with np.load(tmp_path / f) as z:
            ref_keys = sorted(key[len("f%d_" % k):] for key in g if key.startswith("f%d_" % k))
            assert sorted(z.files) == ref_keys
            for key in ref_keys:
                ref = g["f%d_%s" % (k, key)]
                got = z[key]
                if key in ("dt", "cell_size", "np", "m", "h"):
                    np.testing.assert_array_equal(got, ref)
                elif key in ("x", "y", "u", "v"):
                    assert normwise(got - props[key], ref - props[key]) < 1e-4, (f, key)
                else:
                    assert normwise(got, ref) < 1e-4, (f, key)


def test_base5_list_codes_match_oracle():
    """Lists with base-5 cell offsets (used at subdivision 2 above 2^23
    particles), forced on small sets: a 3D lattice RK2 step and a 2D drop
    Euler step against the oracle."""
    _need_gpu()
    import subprocess
    import sys
    code = r'''
import sys
sys.path.insert(0, ".")
import oracle, pysph_gb300
from pysph_gb300 import workloads as W
from tests.golden_util import normwise
api = pysph_gb300.api()
props = W.cube_lattice(32768, seed=4)
s, particles = W.setup_cube(api, props)
assert particles.cell_manager._subdivision() == 2
s.integrator.integrate(1e-4)
pa = particles.arrays[0]
prob = oracle.Problem({"fluid": props}, oracle.cube_ops(), dim=3)
prob.integrate_rk2(1e-4)
for p in ("rho", "p"):
    assert normwise(pa.get(p), prob.arrays["fluid"][p]) < 1e-5, p
for p in ("x", "u", "w"):
    assert normwise(pa.get(p) - props[p], prob.arrays["fluid"][p] - props[p]) < 1e-5, p
props = W.elliptical_drop(dx=0.025, c0=100.0)
s, particles = W.setup_drop(api, props, c0=100.0)
s.integrator.integrate(1e-5)
pa = particles.arrays[0]
prob = oracle.Problem({"fluid": props}, oracle.drop_ops(c0=100.0), dim=2)
prob.integrate_euler(1e-5)
for p in ("rho", "p"):
    assert normwise(pa.get(p), prob.arrays["fluid"][p]) < 1e-5, p
for p in ("x", "y", "u", "v"):
    assert normwise(pa.get(p) - props[p], prob.arrays["fluid"][p] - props[p]) < 1e-5, p
print("ok")
'''
    import os
    # the list-streaming kernels carry the cell-offset codes
    env = dict(os.environ, SPH_WIDE_CODES="1", PYSPH_GB300_SUBDIV="2", PYSPH_GB300_BRICKS="0")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", code], cwd=root, env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr[-3000:]
