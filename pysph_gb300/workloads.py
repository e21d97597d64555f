"""Seeded synthetic particle sets for the standard SPH workloads.

Each builder returns plain NumPy property dictionaries (float64 unless
noted) that can be handed to ``get_particle_array(**props)`` of either this
package or the reference PySPH.  No dataset is read; every input is a
lattice, optionally jittered with ``numpy.random.default_rng(seed)``.

Workloads
---------
* ``elliptical_drop``  -- 2D circular patch, u=-100x, v=100y (the
  elliptical drop of ``examples/elliptical_drop.py``; lattice as in
  ``source/pysph/solver/fluid_solver.py:16-51``).
* ``dam_break``        -- 2D water column with three layers of wall
  particles carrying tangents/normals for ``MonaghanBoundaryForce``.
* ``cube_lattice``     -- 3D jittered lattice filling the unit cube.
* ``drop_batch``       -- many independent elliptical drops of seeded
  radius and spacing.
"""
import math

import numpy as np

FLUID = 0
SOLID = 1


def elliptical_drop(dx=0.025, hdx=1.3, rho0=1.0, c0=1400.0, radius=1.0):
    """Circular patch of fluid on a square lattice.

    Lattice ``mgrid[-1.05:1.05+1e-4:dx]`` scaled by ``radius``; particles
    with ``sqrt(x^2+y^2) - radius > 1e-10`` are dropped (the rule of
    ``fluid_solver.py:37-39``).
    """
    lo = -1.05 * radius
    hi = 1.05 * radius + 1e-4
    x, y = np.mgrid[lo:hi:dx, lo:hi:dx]
    x = x.ravel()
    y = y.ravel()
    keep = np.sqrt(x * x + y * y) - radius <= 1e-10
    x = x[keep].copy()
    y = y[keep].copy()
    n = x.size
    return dict(
        x=x, y=y,
        m=np.full(n, dx * dx * rho0), h=np.full(n, hdx * dx),
        rho=np.full(n, rho0), u=-100.0 * x, v=100.0 * y,
        cs=np.full(n, c0),
    )


def jitter_h(props, frac=0.25, seed=0):
    """Copy of ``props`` with every h scaled by 1 + U(-frac, frac) (seeded):
    smoothing lengths that differ from particle to particle."""
    rng = np.random.default_rng(seed)
    out = dict(props)
    out["h"] = props["h"] * (1.0 + rng.uniform(-frac, frac, size=props["h"].shape))
    return out


def periodic_strip(dx=0.05, nx=20, ny=10, rho0=1.0, c0=10.0, vel_std=1.0, seed=0,
                   rho_jitter=0.01, jitter=0.0):
    """A 2D lattice strip [0, nx dx) x [0, ny dx) meant to be periodic in x
    (domain xmin = 0, xmax = nx dx): points at cell centres (moved by
    U(-jitter, jitter) dx per coordinate), h = 1.3 dx, m = rho0 dx^2,
    velocities N(0, vel_std^2), rho = rho0 (1 + U(-j, j)) and the Tait p, cs
    of that density (gamma = 7) -- a state where every pair term is
    non-trivial.  Seeded."""
    rng = np.random.default_rng(seed)
    xs, ys = np.meshgrid((np.arange(nx) + 0.5) * dx, (np.arange(ny) + 0.5) * dx)
    x = xs.ravel()
    y = ys.ravel()
    n = x.size
    if jitter:
        jr = np.random.default_rng(seed + 1)
        x = x + jr.uniform(-jitter, jitter, n) * dx
        y = y + jr.uniform(-jitter, jitter, n) * dx
    rho = rho0 * (1.0 + rng.uniform(-rho_jitter, rho_jitter, n))
    B = c0 * c0 * rho0 / 7.0
    return dict(x=x, y=y, z=np.zeros(n), u=rng.normal(0.0, vel_std, n),
                v=rng.normal(0.0, vel_std, n), m=np.full(n, rho0 * dx * dx),
                h=np.full(n, 1.3 * dx), rho=rho, p=B * ((rho / rho0) ** 7 - 1.0),
                cs=c0 * (rho / rho0) ** 3)


def circular_patch(dx=0.025, c0=100.0):
    """The reference FluidSolver's circular patch (solver/fluid_solver.py:15-49):
    the square lattice of ``elliptical_drop`` with ``m = dx^2``, ``h = 2 dx``,
    ``rho = 1``, ``p = 0.5 c0^2 (1 - x^2 - y^2)``, ``cs = c0`` and
    ``(u, v) = (-100 x, 100 y)``."""
    props = elliptical_drop(dx=dx, hdx=2.0, rho0=1.0, c0=c0)
    x, y = props["x"], props["y"]
    props["p"] = 0.5 * 1.0 * c0 * c0 * (1.0 - (x * x + y * y))
    return props


def dam_break(dx=0.01, hdx=1.2, rho0=1000.0, column=(1.0, 2.0), tank=(4.0, 3.0),
              layers=3):
    """Water column in a tank with ``layers`` rows of wall particles.

    Fluid particles sit at ``((i+1/2)dx, (j+1/2)dx)`` inside
    ``[0, column[0]] x [0, column[1]]``.  Wall particles sit on the lines
    ``x = -k dx`` (left), ``x = tank[0] + k dx`` (right) and ``y = -k dx``
    (bottom), ``k = 0 .. layers-1``, spaced ``dx`` along the wall, with
    inward unit normals ``(nx, ny)`` and tangents ``(tx, ty)``.

    Returns ``(fluid_props, wall_props)``.
    """
    nx = int(round(column[0] / dx))
    ny = int(round(column[1] / dx))
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    fx = (i.ravel() + 0.5) * dx
    fy = (j.ravel() + 0.5) * dx
    nf = fx.size
    fluid = dict(
        x=fx, y=fy, m=np.full(nf, rho0 * dx * dx), h=np.full(nf, hdx * dx),
        rho=np.full(nf, rho0), cs=np.zeros(nf),
    )

    W, H = tank
    xs, ys, nxs, nys, txs, tys = [], [], [], [], [], []
    nh = int(round(H / dx))
    nw = int(round(W / dx))
    for k in range(layers):
        off = k * dx
        yy = np.arange(0, nh + 1) * dx          # left wall, y in [0, H]
        xs.append(np.full(yy.size, -off)); ys.append(yy)
        nxs.append(np.ones(yy.size)); nys.append(np.zeros(yy.size))
        txs.append(np.zeros(yy.size)); tys.append(np.ones(yy.size))
        xs.append(np.full(yy.size, W + off)); ys.append(yy)   # right wall
        nxs.append(-np.ones(yy.size)); nys.append(np.zeros(yy.size))
        txs.append(np.zeros(yy.size)); tys.append(np.ones(yy.size))
        xx = np.arange(-(layers - 1), nw + layers) * dx       # bottom wall
        xs.append(xx); ys.append(np.full(xx.size, -off))
        nxs.append(np.zeros(xx.size)); nys.append(np.ones(xx.size))
        txs.append(np.ones(xx.size)); tys.append(np.zeros(xx.size))
    wx = np.concatenate(xs)
    wy = np.concatenate(ys)
    nw_ = wx.size
    wall = dict(
        x=wx, y=wy, m=np.full(nw_, rho0 * dx * dx), h=np.full(nw_, hdx * dx),
        rho=np.full(nw_, rho0), cs=np.zeros(nw_),
        nx=np.concatenate(nxs), ny=np.concatenate(nys), nz=np.zeros(nw_),
        tx=np.concatenate(txs), ty=np.concatenate(tys), tz=np.zeros(nw_),
    )
    return fluid, wall


def dam_break_c0(g=9.81, height=2.0):
    """Reference sound speed ``10 sqrt(2 g H)`` of the dam break."""
    return 10.0 * math.sqrt(2.0 * g * height)


def cube_lattice(n, hdx=1.2, rho0=1.0, jitter=0.1, vel_std=0.01, seed=0):
    """3D lattice of ``n1^3`` particles, ``n1 = round(n^(1/3))``, filling the unit cube.

    Positions ``(i+1/2)dx`` plus uniform jitter in ``[-jitter dx, jitter dx]``,
    velocities ``N(0, vel_std^2)`` per component, ``m = rho0 dx^3``,
    ``h = hdx dx``.
    """
    n1 = int(round(n ** (1.0 / 3.0)))
    dx = 1.0 / n1
    rng = np.random.default_rng(seed)
    idx = np.arange(n1)
    # x fastest, so consecutive particles are x-neighbours
    z, y, x = np.meshgrid(idx, idx, idx, indexing="ij")
    N = n1 ** 3
    pos = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1).astype(np.float64)
    pos = (pos + 0.5) * dx + rng.uniform(-jitter * dx, jitter * dx, size=(N, 3))
    vel = rng.normal(0.0, vel_std, size=(N, 3))
    return dict(
        x=pos[:, 0].copy(), y=pos[:, 1].copy(), z=pos[:, 2].copy(),
        u=vel[:, 0].copy(), v=vel[:, 1].copy(), w=vel[:, 2].copy(),
        m=np.full(N, rho0 * dx ** 3), h=np.full(N, hdx * dx),
        rho=np.full(N, rho0), cs=np.zeros(N),
    )


def drop_batch(count=256, seed=0, rmin=0.5, rmax=1.5, dxmin=0.01, dxmax=0.04,
               hdx=1.3, rho0=1.0, c0=1400.0, max_particles=None):
    """``count`` independent elliptical drops of seeded radius and spacing.

    With ``max_particles`` set, the spacing of a drop is raised until it
    holds at most that many particles (used to bound test sizes).
    """
    rng = np.random.default_rng(seed)
    radii = rng.uniform(rmin, rmax, size=count)
    dxs = rng.uniform(dxmin, dxmax, size=count)
    out = []
    for r, dx in zip(radii, dxs):
        if max_particles is not None:
            est = math.pi * r * r / (dx * dx)
            if est > max_particles:
                dx = r * math.sqrt(math.pi / max_particles)
        out.append(elliptical_drop(dx=dx, hdx=hdx, rho0=rho0, c0=c0, radius=r))
    return out


# ---------------------------------------------------------------------------
# Solver recipes.  ``api`` is a namespace with ``base``, ``sph`` and
# ``solver`` modules: either this package's or the reference PySPH's, so the
# same recipe builds the same operation list on both sides.
# ---------------------------------------------------------------------------

def _integrator(api, name):
    return {"euler": api.solver.EulerIntegrator,
            "rk2": api.solver.RK2Integrator,
            "rk4": api.solver.RK4Integrator,
            "pc": api.solver.PredictorCorrectorIntegrator,
            "leapfrog": api.solver.LeapFrogIntegrator}[name]


def setup_drop(api, props, c0=1400.0, rho0=1.0, alpha=0.01, beta=0.0, eps=0.5,
               integrator="euler", name="fluid", variable_h=False, periodic_domain=None,
               adke=None):
    """Elliptical drop operations: SPHRho, Tait, PGrad, Monaghan AV,
    position stepping and XSPH, in that order (2D).  ``variable_h`` makes
    the neighbour relation symmetric (``Particles(variable_h=True)``).
    ``adke=(h0, k, eps)`` puts the ADKE pilot density and smoothing-length
    update first, as examples/shock-tube/sigalotti_shock_tube.py:44-56 does
    (``props`` needs ``rhop``)."""
    base, sph, solver = api.base, api.sph, api.solver
    Fluid = base.ParticleType.Fluid
    pa = base.get_particle_array(name=name, type=Fluid, **props)
    particles = base.Particles(arrays=[pa], variable_h=variable_h,
                               periodic_domain=periodic_domain)
    s = solver.Solver(dim=2, integrator_type=_integrator(api, integrator))
    if adke is not None:
        h0, k, e = adke
        s.add_operation(solver.SPHOperation(
            sph.ADKEPilotRho.withargs(h0=h0), on_types=[Fluid], from_types=[Fluid],
            updates=["rhop"], id="adke_rho"))
        s.add_operation(solver.SPHOperation(
            sph.ADKESmoothingUpdate.withargs(h0=h0, k=k, eps=e), on_types=[Fluid],
            updates=["h"], id="adke"))
    s.add_operation(solver.SPHOperation(
        sph.SPHRho.withargs(), on_types=[Fluid], from_types=[Fluid],
        updates=["rho"], id="density"))
    s.add_operation(solver.SPHOperation(
        sph.TaitEquation.withargs(co=c0, ro=rho0), on_types=[Fluid],
        updates=["p", "cs"], id="eos"))
    s.add_operation(solver.SPHIntegration(
        sph.SPHPressureGradient.withargs(dim=2), on_types=[Fluid],
        from_types=[Fluid], updates=["u", "v"], id="pgrad"))
    s.add_operation(solver.SPHIntegration(
        sph.MonaghanArtificialVsicosity.withargs(alpha=alpha, beta=beta),
        on_types=[Fluid], from_types=[Fluid], updates=["u", "v", "w"],
        id="avisc"))
    s.add_operation_step([Fluid])
    s.add_operation_xsph(eps=eps)
    s.setup_integrator(particles)
    return s, particles


def setup_fluid_solver(api, props, c0=100.0, ro=1.0, alpha=0.01, beta=0.0, eps=0.1,
                       integrator="rk2"):
    """The reference FluidSolver's operations (solver/fluid_solver.py:51-83):
    Tait, continuity density rate, MomentumEquation (eta stored, 0.1),
    position stepping and XSPH (2D)."""
    base, sph, solver = api.base, api.sph, api.solver
    Fluid = base.ParticleType.Fluid
    pa = base.get_particle_array(name="fluid", type=Fluid, **props)
    particles = base.Particles(arrays=[pa])
    s = solver.Solver(dim=2, integrator_type=_integrator(api, integrator))
    s.add_operation(solver.SPHOperation(
        sph.TaitEquation.withargs(co=c0, ro=ro), on_types=[Fluid],
        updates=["p", "cs"], id="eos"))
    s.add_operation(solver.SPHIntegration(
        sph.SPHDensityRate.withargs(hks=False), from_types=[Fluid], on_types=[Fluid],
        updates=["rho"], id="density"))
    s.add_operation(solver.SPHIntegration(
        sph.MomentumEquation.withargs(alpha=alpha, beta=beta, hks=False),
        from_types=[Fluid], on_types=[Fluid], updates=["u", "v", "w"], id="mom"))
    s.add_operation_step([Fluid])
    s.add_operation_xsph(eps=eps, hks=False)
    s.setup_integrator(particles)
    return s, particles


def setup_dam_break(api, fluid_props, wall_props, dx, c0, rho0=1000.0,
                    alpha=0.1, beta=0.0, g=-9.81, integrator="rk2"):
    """Dam-break operations: Tait, SPHRho (fluid<-fluid), PGrad and Monaghan
    AV (fluid<-fluid), Monaghan boundary force (fluid<-solid), gravity and
    position stepping (2D)."""
    base, sph, solver = api.base, api.sph, api.solver
    Fluid = base.ParticleType.Fluid
    Solid = base.ParticleType.Solid
    fluid = base.get_particle_array(name="fluid", type=Fluid, **fluid_props)
    wall = base.get_particle_array(name="boundary", type=Solid, **wall_props)
    particles = base.Particles(arrays=[fluid, wall])
    s = solver.Solver(dim=2, integrator_type=_integrator(api, integrator))
    s.add_operation(solver.SPHOperation(
        sph.TaitEquation.withargs(co=c0, ro=rho0), on_types=[Fluid],
        updates=["p", "cs"], id="eos"))
    s.add_operation(solver.SPHOperation(
        sph.SPHRho.withargs(), on_types=[Fluid], from_types=[Fluid],
        updates=["rho"], id="density"))
    s.add_operation(solver.SPHIntegration(
        sph.SPHPressureGradient.withargs(dim=2), on_types=[Fluid],
        from_types=[Fluid], updates=["u", "v"], id="pgrad"))
    s.add_operation(solver.SPHIntegration(
        sph.MonaghanArtificialVsicosity.withargs(alpha=alpha, beta=beta),
        on_types=[Fluid], from_types=[Fluid], updates=["u", "v", "w"],
        id="avisc"))
    s.add_operation(solver.SPHIntegration(
        sph.MonaghanBoundaryForce.withargs(delp=dx), on_types=[Fluid],
        from_types=[Solid], updates=["u", "v", "w"], id="bforce"))
    s.add_operation(solver.SPHIntegration(
        sph.GravityForce.withargs(gy=g), on_types=[Fluid],
        updates=["u", "v", "w"], id="gravity"))
    s.add_operation_step([Fluid])
    s.setup_integrator(particles)
    return s, particles


def setup_cube(api, props, c0=1.0, rho0=1.0, alpha=0.1, beta=0.0,
               integrator="rk2"):
    """3D throughput operations: SPHRho, Tait, PGrad, Monaghan AV and
    position stepping."""
    base, sph, solver = api.base, api.sph, api.solver
    Fluid = base.ParticleType.Fluid
    pa = base.get_particle_array(name="fluid", type=Fluid, **props)
    particles = base.Particles(arrays=[pa])
    s = solver.Solver(dim=3, integrator_type=_integrator(api, integrator))
    s.add_operation(solver.SPHOperation(
        sph.SPHRho.withargs(), on_types=[Fluid], from_types=[Fluid],
        updates=["rho"], id="density"))
    s.add_operation(solver.SPHOperation(
        sph.TaitEquation.withargs(co=c0, ro=rho0), on_types=[Fluid],
        updates=["p", "cs"], id="eos"))
    s.add_operation(solver.SPHIntegration(
        sph.SPHPressureGradient.withargs(dim=3), on_types=[Fluid],
        from_types=[Fluid], updates=["u", "v", "w"], id="pgrad"))
    s.add_operation(solver.SPHIntegration(
        sph.MonaghanArtificialVsicosity.withargs(alpha=alpha, beta=beta),
        on_types=[Fluid], from_types=[Fluid], updates=["u", "v", "w"],
        id="avisc"))
    s.add_operation_step([Fluid])
    s.setup_integrator(particles)
    return s, particles
