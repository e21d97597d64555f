"""Generate the golden fixtures in this folder from the reference PySPH.

Runs the compat-patched reference build (``oracle/_ref/src``, made by
``python oracle/build_ref.py``) on seeded synthetic inputs and stores, per
fixture, the inputs, the per-evaluation outputs of every calc, the neighbour
sets and the state after the step.  The fixtures are what the parity tests
compare the GPU path (and the C restatement in ``oracle/``) against.

Usage: ``python tests/golden/make_golden.py`` (needs the reference build; it
is not run by the tests).
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref", "src"))

import pysph.base.api as rbase  # noqa: E402  (reference)
import pysph.sph.api as rsph  # noqa: E402
import pysph.solver.api as rsolver  # noqa: E402

from pysph_gb300 import workloads as W  # noqa: E402

REF = types.SimpleNamespace(base=rbase, sph=rsph, solver=rsolver)

STATE = ("x", "y", "z", "u", "v", "w")
EVAL_PROPS = ("x", "y", "z", "u", "v", "w", "rho", "p", "cs")


def neighbours_csr(particles, src, dst, radius_scale=2.0):
    """Neighbour lists (reference order, self last) as CSR arrays."""
    loc = particles.nnps_manager.get_neighbor_particle_locator(src, dst, radius_scale)
    offs = [0]
    idx = []
    for i in range(dst.get_number_of_particles()):
        nb = loc.py_get_nearest_particles(i).get_npy_array().copy()
        idx.append(nb)
        offs.append(offs[-1] + nb.size)
    return np.asarray(offs, np.int64), np.concatenate(idx).astype(np.int32)


def run_step(s, particles, dt, out, nbr_pairs=()):
    """One integrator step, snapshotting every evaluation."""
    integ = s.integrator
    arrays = particles.arrays
    for pa in arrays:
        for p in pa.properties:
            if p in ("tag", "group", "local", "idx") or p.startswith("_"):
                continue
            out["in_%s_%s" % (pa.name, p)] = pa.get(p).copy()
    for (si, di) in nbr_pairs:
        o, ix = neighbours_csr(particles, arrays[si], arrays[di])
        out["nbr_%s_%s_offsets" % (arrays[di].name, arrays[si].name)] = o
        out["nbr_%s_%s_index" % (arrays[di].name, arrays[si].name)] = ix

    counter = [0]
    orig_eval = integ.eval

    def eval_and_record(calcs):
        e = counter[0] + 1
        kn = "k%d" % integ.cstep
        for pa in arrays:
            for p in STATE:
                out["eval%d_pre_%s_%s" % (e, pa.name, p)] = pa.get(p).copy()
        orig_eval(calcs)
        for pa in arrays:
            for p in ("rho", "p", "cs"):
                out["eval%d_%s_%s" % (e, pa.name, p)] = pa.get(p).copy()
        for calc in calcs:
            if calc.integrates:
                pa = arrays[calc.dnum]
                names = calc.dst_writes[kn]
                for j, upd in enumerate(calc.updates):
                    out["eval%d_k_%s_%s" % (e, calc.id, upd)] = pa.get(names[j]).copy()
        counter[0] += 1

    integ.eval = eval_and_record
    integ.integrate(dt)
    integ.eval = orig_eval
    for pa in arrays:
        for p in STATE + ("rho", "p", "cs"):
            out["out_%s_%s" % (pa.name, p)] = pa.get(p).copy()
    out["n_evals"] = np.int64(counter[0])
    out["dt"] = np.float64(dt)


def fixture_kernel():
    """Cubic-spline W and grad W on a grid of distances, h and dimensions."""
    out = {}
    rs = np.concatenate([np.linspace(0.0, 2.2, 45), [1e-15, 0.5, 1.0, 2.0, 1.0 - 1e-12, 2.0 - 1e-12]])
    for dim in (1, 2, 3):
        k = rbase.CubicSplineKernel(dim=dim)
        for h in (0.1, 0.37, 1.0):
            w = np.zeros(rs.size)
            g = np.zeros((rs.size, 3))
            pa = rbase.Point(0.0, 0.0, 0.0)
            for n, r in enumerate(rs):
                # points along a skew direction so every component is exercised
                d = np.array([0.6, -0.48, 0.64])[:dim]
                d = d / np.linalg.norm(d)
                q = np.zeros(3)
                q[:dim] = d * r * h
                pb = rbase.Point(*q)
                w[n] = k.py_function(pa, pb, h)
                gp = rbase.Point()
                k.py_gradient(pa, pb, h, gp)
                g[n] = (gp.x, gp.y, gp.z)
            out["w_d%d_h%g" % (dim, h)] = w
            out["g_d%d_h%g" % (dim, h)] = g
    out["r_over_h"] = rs
    return out


def fixture_square4():
    """Four particles on a unit square (the reference's SPH function tests)."""
    out = {}
    x = np.array([0, 0, 1, 1], np.float64)
    y = np.array([0, 1, 1, 0], np.float64)
    u = np.array([1, 0, 0, -1], np.float64)
    p = np.array([0, 0, 1, 1], np.float64)
    pa = rbase.get_particle_array(name="test", x=x, y=y, z=np.zeros(4), m=np.ones(4),
                                  u=u, p=p, cs=np.ones(4),
                                  tmpx=np.zeros(4), tmpy=np.zeros(4), tmpz=np.zeros(4))
    particles = rbase.Particles(arrays=[pa])
    kern = rbase.CubicSplineKernel(dim=2)
    for name, fn, ups in (
            ("rho", rsph.SPHRho.withargs(), ["tmpx"]),
            ("pgrad", rsph.SPHPressureGradient.withargs(dim=2), ["tmpx", "tmpy"]),
            ("avisc", rsph.MonaghanArtificialVsicosity.withargs(alpha=1.0, beta=1.0),
             ["tmpx", "tmpy", "tmpz"]),
            ("xsph", rsph.XSPHCorrection.withargs(eps=0.5, dim=2), ["tmpx", "tmpy"])):
        func = fn.get_func(pa, pa)
        calc = rsph.SPHCalc(particles, [pa], pa, kern, [func], ups)
        calc.sph(*ups)
        for k, upn in enumerate(ups):
            out["%s_%d" % (name, k)] = pa.get(upn).copy()
    for p_ in ("x", "y", "u", "p", "m", "h", "rho", "cs"):
        out["in_" + p_] = pa.get(p_).copy()
    return out


def fixture_drop(steps=1, dx=0.025):
    props = W.elliptical_drop(dx=dx)
    s, particles = W.setup_drop(REF, props)
    out = {}
    run_step(s, particles, 1e-5, out, nbr_pairs=[(0, 0)])
    for _ in range(steps - 1):
        s.integrator.integrate(1e-5)
    if steps > 1:
        pa = particles.arrays[0]
        for p in ("x", "y", "u", "v", "rho", "p", "cs"):
            out["final_%s" % p] = pa.get(p).copy()
        out["steps"] = np.int64(steps)
    return out


def fixture_dam(dx=0.04):
    fl, wl = W.dam_break(dx=dx)
    c0 = W.dam_break_c0()
    s, particles = W.setup_dam_break(REF, fl, wl, dx=dx, c0=c0)
    out = {"dx": np.float64(dx), "c0": np.float64(c0)}
    run_step(s, particles, 1e-4, out, nbr_pairs=[(0, 0), (1, 0)])
    return out


def fixture_fluid(dx=0.05):
    """The reference FluidSolver recipe (continuity + MomentumEquation) on
    its circular patch, one RK2 step."""
    props = W.circular_patch(dx=dx)
    s, particles = W.setup_fluid_solver(REF, props)
    out = {}
    run_step(s, particles, 1e-4, out, nbr_pairs=[(0, 0)])
    return out


def fixture_square4_momentum():
    """MomentumEquation (alpha = beta = 1, eta = 0.1) and SPHDensityRate on
    the four-particle square of the reference's function tests."""
    out = {}
    x = np.array([0, 0, 1, 1], np.float64)
    y = np.array([0, 1, 1, 0], np.float64)
    u = np.array([1, 0, 0, -1], np.float64)
    v = np.array([0, 1, -1, 0], np.float64)
    p = np.array([0, 0, 1, 1], np.float64)
    pa = rbase.get_particle_array(name="test", x=x, y=y, z=np.zeros(4), m=np.ones(4),
                                  u=u, v=v, p=p, cs=np.ones(4),
                                  tmpx=np.zeros(4), tmpy=np.zeros(4), tmpz=np.zeros(4))
    particles = rbase.Particles(arrays=[pa])
    kern = rbase.CubicSplineKernel(dim=2)
    for name, fn, ups in (
            ("momentum", rsph.MomentumEquation.withargs(alpha=1.0, beta=1.0, eta=0.1),
             ["tmpx", "tmpy", "tmpz"]),
            ("drho", rsph.SPHDensityRate.withargs(), ["tmpx"])):
        func = fn.get_func(pa, pa)
        calc = rsph.SPHCalc(particles, [pa], pa, kern, [func], ups)
        calc.sph(*ups)
        for k, upn in enumerate(ups):
            out["%s_%d" % (name, k)] = pa.get(upn).copy()
    for p_ in ("x", "y", "u", "v", "p", "m", "h", "rho", "cs"):
        out["in_" + p_] = pa.get(p_).copy()
    return out


def fixture_cube(n=4096, integrator="rk2"):
    props = W.cube_lattice(n)
    s, particles = W.setup_cube(REF, props, integrator=integrator)
    out = {}
    run_step(s, particles, 1e-4, out, nbr_pairs=[(0, 0)])
    return out


def fixture_drop_integrator(integrator, dx=0.05, steps=3):
    """The elliptical drop stepped by another integrator: the first step
    recorded evaluation by evaluation, then the state after ``steps``."""
    props = W.elliptical_drop(dx=dx)
    s, particles = W.setup_drop(REF, props, integrator=integrator)
    out = {}
    run_step(s, particles, 1e-5, out, nbr_pairs=[(0, 0)])
    for _ in range(steps - 1):
        s.integrator.integrate(1e-5)
    pa = particles.arrays[0]
    for p in ("x", "y", "u", "v", "rho", "p", "cs"):
        out["final_%s" % p] = pa.get(p).copy()
    out["steps"] = np.int64(steps)
    return out


def fixture_fluid_integrator(integrator, dx=0.05, steps=3):
    """The FluidSolver recipe (integrated density) under another integrator."""
    props = W.circular_patch(dx=dx)
    s, particles = W.setup_fluid_solver(REF, props, integrator=integrator)
    out = {}
    run_step(s, particles, 1e-4, out, nbr_pairs=[(0, 0)])
    for _ in range(steps - 1):
        s.integrator.integrate(1e-4)
    pa = particles.arrays[0]
    for p in ("x", "y", "u", "v", "rho", "p", "cs"):
        out["final_%s" % p] = pa.get(p).copy()
    out["steps"] = np.int64(steps)
    return out


def fixture_drop_varh(dx=0.05):
    """The elliptical drop with per-particle h (U(-25 %, 25 %) about 1.3 dx)
    and Particles(variable_h=True): symmetric neighbour lists
    (VarHNbrParticleLocator) and one Euler step."""
    props = W.jitter_h(W.elliptical_drop(dx=dx))
    s, particles = W.setup_drop(REF, props, variable_h=True)
    out = {}
    run_step(s, particles, 1e-5, out, nbr_pairs=[(0, 0)])
    return out


def fixture_periodic(dx=0.05, nx=20, ny=10):
    """Particles(periodic_domain=PeriodicDomain(0, nx dx)) on a lattice strip:
    the ghost copies the reference appends (cell.pyx:1277-1376), the
    neighbour lists over real and ghost particles, and each pair function
    evaluated on the initial state (where the ghosts still carry their
    originals' state; a calc zeroes them as non-LocalReal destinations)."""
    props = W.periodic_strip(dx=dx, nx=nx, ny=ny)
    n = len(props["x"])
    extra = {k: np.zeros(n) for k in ("tmpx", "tmpy", "tmpz")}
    pa = rbase.get_particle_array(name="fluid", type=rbase.ParticleType.Fluid,
                                  **props, **extra)
    dom = rbase.PeriodicDomain(xmin=0.0, xmax=nx * dx)
    particles = rbase.Particles(arrays=[pa], periodic_domain=dom)
    out = {"xmin": np.float64(0.0), "xmax": np.float64(nx * dx), "n_real": np.int64(n)}
    for p_ in props:
        out["in_" + p_] = props[p_].copy()
    xa = pa.get("x", only_real_particles=False)
    ya = pa.get("y", only_real_particles=False)
    ng = len(xa) - n
    origin = np.full(ng, -1, np.int64)
    shift = np.zeros(ng)
    L = nx * dx
    for g in range(ng):
        for s in (L, -L):
            hit = np.nonzero((xa[:n] + s == xa[n + g]) & (ya[:n] == ya[n + g]))[0]
            if hit.size:
                origin[g], shift[g] = hit[0], s
                break
    assert (origin >= 0).all()
    out["ghost_origin"] = origin
    out["ghost_shift"] = shift
    o, ix = neighbours_csr(particles, pa, pa)
    out["nbr_offsets"] = o[: n + 1]
    out["nbr_index"] = ix[: o[n]]
    kern = rbase.CubicSplineKernel(dim=2)
    for name, fn, ups in (
            ("pgrad", rsph.SPHPressureGradient.withargs(dim=2), ["tmpx", "tmpy"]),
            ("avisc", rsph.MonaghanArtificialVsicosity.withargs(alpha=1.0, beta=1.0),
             ["tmpx", "tmpy", "tmpz"]),
            ("xsph", rsph.XSPHCorrection.withargs(eps=0.5, dim=2), ["tmpx", "tmpy"]),
            ("rho", rsph.SPHRho.withargs(), ["tmpx"])):
        calc = rsph.SPHCalc(particles, [pa], pa, kern, [fn.get_func(pa, pa)], ups)
        calc.sph(*ups)
        for k, upn in enumerate(ups):
            out["%s_%d" % (name, k)] = pa.get(upn)[:n].copy()
    return out


ADKE = {"h0_dx": 1.2, "k": 1.0, "eps": 0.5, "g1": 0.2, "g2": 0.4}


def fixture_adke(dx=0.05):
    """ADKE (Sigalotti's adaptive kernel estimation, sph/funcs/adke_funcs.pyx)
    on the elliptical drop with per-particle h, a seeded velocity
    perturbation and Particles(variable_h=True), each function through an
    SPHCalc as the reference's shock-tube example chains them: the pilot
    density at the fixed h0, the smoothing-length update from it (the calc
    marks the array dirty and re-bins), then the velocity divergence and the
    conduction coefficient on the new h; with the neighbour lists before and
    after the update."""
    props = W.jitter_h(W.elliptical_drop(dx=dx, c0=100.0))
    n = len(props["x"])
    rng = np.random.default_rng(11)
    props["u"] = props["u"] + rng.normal(0.0, 5.0, n)
    props["v"] = props["v"] + rng.normal(0.0, 5.0, n)
    extra = {k: np.zeros(n) for k in ("rhop", "div", "q", "tmpx", "tmpy")}
    pa = rbase.get_particle_array(name="fluid", type=rbase.ParticleType.Fluid,
                                  **props, **extra)
    particles = rbase.Particles(arrays=[pa], variable_h=True)
    kern = rbase.CubicSplineKernel(dim=2)
    h0 = ADKE["h0_dx"] * dx
    out = {"h0": np.float64(h0), "k": np.float64(ADKE["k"]), "eps": np.float64(ADKE["eps"]),
           "g1": np.float64(ADKE["g1"]), "g2": np.float64(ADKE["g2"])}
    for p_ in props:
        out["in_" + p_] = np.asarray(props[p_]).copy()
    o, ix = neighbours_csr(particles, pa, pa)
    out["nbr0_offsets"], out["nbr0_index"] = o, ix

    def run(fn, ups):
        calc = rsph.SPHCalc(particles, [pa], pa, kern, [fn.get_func(pa, pa)], ups)
        calc.sph(*ups)

    run(rsph.ADKEPilotRho.withargs(h0=h0), ["rhop"])
    out["rhop"] = pa.get("rhop").copy()
    run(rsph.ADKESmoothingUpdate.withargs(h0=h0, k=ADKE["k"], eps=ADKE["eps"]), ["h"])
    out["h_new"] = pa.get("h").copy()
    o, ix = neighbours_csr(particles, pa, pa)
    out["nbr1_offsets"], out["nbr1_index"] = o, ix
    # three outputs: the class keeps SPHFunction's num_outputs (a one-update
    # calc, as in examples/shock-tube/sigalotti_shock_tube.py, raises)
    run(rsph.VelocityDivergence.withargs(), ["div", "tmpx", "tmpy"])
    out["div"] = pa.get("div").copy()
    out["div_1"] = pa.get("tmpx").copy()
    out["div_2"] = pa.get("tmpy").copy()
    run(rsph.ADKEConductionCoeffUpdate.withargs(g1=ADKE["g1"], g2=ADKE["g2"]), ["q"])
    out["q"] = pa.get("q").copy()
    return out


def fixture_drop_output(dx=0.1, steps=3):
    """Solver.solve of the drop with output every step (solver.py:457-538):
    the names of the .npz files it writes and their contents."""
    import tempfile
    props = W.elliptical_drop(dx=dx)
    s, particles = W.setup_drop(REF, props)
    s.set_time_step(1e-5)
    s.set_final_time(steps * 1e-5 * (1 - 1e-9))
    s.set_print_freq(1)
    # the reference's Solver reads detailed_output, which only this setter
    # creates (solver.py:520)
    s.set_output_printing_level(False)
    out = {}
    with tempfile.TemporaryDirectory() as d:
        s.set_output_directory(d)
        s.set_output_fname("drop")
        s.solve()
        names = sorted(os.listdir(d))
        out["files"] = np.array(names)
        for k, f in enumerate(names):
            with np.load(os.path.join(d, f)) as z:
                for key in z.files:
                    out["f%d_%s" % (k, key)] = z[key]
    for p_ in props:
        out["in_" + p_] = np.asarray(props[p_]).copy()
    return out


def main():
    fixtures = {
        "kernel": fixture_kernel,
        "square4": fixture_square4,
        "drop_step": lambda: fixture_drop(1),
        "drop_traj10": lambda: fixture_drop(10),
        "dam_step": fixture_dam,
        "cube_step": fixture_cube,
        "fluid_step": fixture_fluid,
        "square4_momentum": fixture_square4_momentum,
        "drop_rk4": lambda: fixture_drop_integrator("rk4"),
        "drop_pc": lambda: fixture_drop_integrator("pc"),
        "fluid_rk4": lambda: fixture_fluid_integrator("rk4"),
        "fluid_pc": lambda: fixture_fluid_integrator("pc"),
        "cube_leapfrog": lambda: fixture_cube(1000, "leapfrog"),
        "drop_varh": fixture_drop_varh,
        "periodic": fixture_periodic,
        "drop_output": fixture_drop_output,
        "adke": fixture_adke,
    }
    only = sys.argv[1:]
    if only:
        fixtures = {k: v for k, v in fixtures.items() if k in only}
    for name, fn in fixtures.items():
        data = fn()
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **data)
        print("wrote", path, os.path.getsize(path) // 1024, "KiB")


if __name__ == "__main__":
    main()
